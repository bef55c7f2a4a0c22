"""Benchmark of the Barnes-Hut step on GB300: particle-updates/s.

Default workload (the largest configuration on one GPU, at the tree depth the
reference uses): N = 16,777,216 particles uniform in a unit cube (seeded
Gaussian velocities, sigma 0.1; log-normal masses, sigma 0.5, total 1),
PHYSICAL preset, plain FP32, theta = 0.7, eps = 0.001, dt = 1e-3, lbits = 6
(the reference's 7 layers, MortonCode.metal:43-50). One step = bbox,
encode, sort, Morton reorder, tree topology, per-layer aggregation, the
group walk and its evaluation with the fused kick-drift.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload c1|c2|c3|c4|c5|ref] [--form plain|precision]

`value` is the device-timed throughput with inputs resident in HBM (CUDA
events on the context's stream around each step, L2 flushed before every
timed step). `e2e` is the same metric through the C ABI with host buffers:
each step uploads PositionMass/VelocityRadius from pinned host memory, steps
and downloads them, the transfers pipelined with the steps
(astro_upload_async / astro_download_async). Extra keys of the default line: the same workload with
all 21 bits per axis (63-bit keys) and in the precision form, and the
metric's comparison on the batching workload (256 Plummer systems): plain
FP32 batched, precision + batched, and the systems stepped one at a time.
`--impl reference` times the CPU restatement of the reference kernels
(oracle/, OpenMP over all host cores) on the same workload within a time
budget. Under torchrun every rank runs an independent replica of a
single-system workload (one tree per step must be globally consistent), and
the batching workload's systems are sharded over the ranks in contiguous
ranges balanced by N log N (astro_gb300.shard; no exchange); rank 0 prints
the line with the max time over ranks.
"""
from __future__ import annotations

import argparse
import dataclasses
import datetime
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

from astro_gb300.workloads import WORKLOADS  # noqa: E402  (no CUDA needed to import)

METRIC = "particle-updates/s per GB300 step (plain FP32 vs precision+batched) at stated FP64 error"
UNIT = "particle-updates/s"
# Flops per interaction: 20 for a softened particle-particle or monopole term
# (the GPU Gems 3 ch. 31 convention); 50 for a cell with its quadrupole term
# (the monopole's 20 plus Qd (15), d.Qd (5), the radial factor (4) and the
# two vector updates (6), counting an FMA as 2).
FLOPS_PER_INTERACTION = 20
FLOPS_PER_QUAD_CELL = 50
# A far node's expansion about its walk's centre: 350 flops once per walk
# (the field, its 6 first and 10 second derivatives from the monopole and
# quadrupole, and their 19 sums; group_far_kernel, timed with the
# evaluation), and 70 per particle of a group with far nodes to evaluate
# the expansion (3 x (J rho, H rho rho, sums)).
FLOPS_PER_FAR_NODE = 350
FLOPS_PER_FAR_EVAL = 70
L2_FLUSH_BYTES = 256 << 20  # larger than the 129 MB L2
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of
# the kernels the roofline times for (workload, form, lbits): its "traffic".
# C5 at lbits 6: one ncu capture of each of the same kernels on the same law
# at 2,097,152 particles (lbits 5, 64 particles per leaf as at full size;
# cold cache): the evaluation 228.44 MB and the far-node sums 51.15 MB,
# scaled by the particle count (x8).
NCU_EVAL_DRAM_BYTES: dict = {("c5", "plain", 6): (228.444672e6 + 51.145472e6) * 8}


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="c5",
                    help="c1..c5: PHYSICAL workloads; ref: the reference's own scene")
    ap.add_argument("--form", choices=["plain", "precision"], default="plain")
    ap.add_argument("--n", type=int, default=None,
                    help="particles of a single-system workload (smaller cases for profiling)")
    # Launch knobs: unset ones come from the autotuner's file for the
    # workload, form and tree depth (astro_gb300/tuned.json), else the
    # preset defaults. The tree depth defaults to the workload's quoted one.
    ap.add_argument("--lbits", type=int, default=None)
    ap.add_argument("--bucket", type=int, default=None)
    ap.add_argument("--warps", type=int, default=None)
    ap.add_argument("--group-size", type=int, default=None)
    ap.add_argument("--sort-variant", type=int, default=None)
    ap.add_argument("--delta-weight", type=float, default=None,
                    help="w of the opening radius size/theta + w |com - cell centre|")
    ap.add_argument("--far-ratio", type=float, default=None,
                    help="group walk: nodes further than (group radius) / r from the group's "
                         "centre are summed through one expansion per group (0: none)")
    ap.add_argument("--walk-frontier", type=int, default=None, choices=[0, 1],
                    help="group walk frontier: 0 = runs of consecutive nodes, 1 = node list")
    ap.add_argument("--no-tuned", action="store_true", help="ignore the autotuner's file")
    ap.add_argument("--theta", type=float, default=0.7)
    ap.add_argument("--persistent", action="store_true")
    ap.add_argument("--walk", choices=["group", "particle"], default="group")
    ap.add_argument("--monopole", action="store_true",
                    help="the reference's monopole-only cells and size/theta opening test")
    ap.add_argument("--error-samples", type=int, default=2048)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--cpu-threads", type=int, default=0,
                    help="host threads of the CPU restatement (0: all cores)")
    ap.add_argument("--reference-seconds", type=float, default=120.0,
                    help="--impl reference: time budget of the timed CPU steps")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the extra configurations of the default line")
    return ap.parse_args(argv)


def workload(args):
    """The workload of --workload, with --n particles when given."""
    w = WORKLOADS[args.workload]
    n = getattr(args, "n", None)
    if n is not None:
        if w.generator in ("batch", "reference_scene"):
            raise SystemExit("--n applies to the single-system PHYSICAL workloads")
        w = dataclasses.replace(w, n=n)
    return w


CLIMB_MIN_NODES = 32768  # build.cu: layers of at least this capacity get a launch each


def kernels_per_step(key_bits: int, layer_sizes, preset: str = "physical") -> int:
    """This library's kernel launches in one step. PHYSICAL: bbox, setup,
    encode, sort histogram + one pass per 8 key bits, Morton reorder,
    topology, the per-layer aggregations below the climb + the climbing
    one, the group walk and its evaluation (9 + passes + per-layer
    aggregations). REFERENCE: encode, sort histogram + passes, topology,
    aggregations, traversal, lights snapshot + lighting, integrate (8 +
    passes + per-layer aggregations)."""
    passes = (key_bits + 7) // 8
    l0 = 0
    while l0 + 1 < len(layer_sizes) and layer_sizes[l0] >= CLIMB_MIN_NODES:
        l0 += 1
    return (9 if preset == "physical" else 8) + passes + l0


def walk_flags(args, L, flags):
    """Traversal flags: the preset's defaults adjusted by --walk/--monopole."""
    if args.walk == "particle":
        flags |= L.FLAG_PER_PARTICLE
    if args.monopole:
        flags &= ~(L.FLAG_QUADRUPOLE | L.FLAG_OPEN_DELTA)
    if args.persistent:
        flags |= L.FLAG_PERSISTENT
    return flags


def quoted_lbits(args):
    """The tree depth the line is quoted at: --lbits, else the workload's
    quoted depth (c5: the reference's 7 layers), else None (tuned)."""
    if args.lbits is not None:
        return args.lbits, "command line"
    w = WORKLOADS[args.workload]
    if w.quoted_lbits is not None:
        return w.quoted_lbits, "the workload's quoted depth"
    return None, None


def knobs(args):
    """Launch knobs: command line, else the tuned file (the entry searched at
    the quoted tree depth when there is one), else the defaults."""
    tuned = {}
    lbits, lsrc = quoted_lbits(args)
    if not args.no_tuned:
        from astro_gb300 import autotune

        res = autotune.load()
        key = autotune.result_key(args.workload, args.form, lbits)
        entry = res.get(key) or res.get(autotune.result_key(args.workload, args.form))
        tuned = (entry or {}).get("knobs", {})
    default = {"lbits": WORKLOADS[args.workload].lbits, "bucket": 16, "block_warps": 0,
               "group_size": 0, "sort_variant": 0, "open_delta_weight": 1.0, "far_ratio": 0.0,
               "walk_frontier": 0}
    given = {"lbits": args.lbits, "bucket": args.bucket, "block_warps": args.warps,
             "group_size": args.group_size, "sort_variant": args.sort_variant,
             "open_delta_weight": args.delta_weight, "far_ratio": args.far_ratio,
             "walk_frontier": args.walk_frontier}
    out, source = {}, {}
    for k in default:
        if given[k] is not None:
            out[k], source[k] = given[k], "command line"
        elif k == "lbits" and lbits is not None:
            out[k], source[k] = lbits, lsrc
        elif k in tuned:
            out[k], source[k] = tuned[k], "autotuner"
        else:
            out[k], source[k] = default[k], "default"
    return out, source


def make_params(args, L, default_params):
    w = workload(args)
    form = L.FORM_PRECISION if args.form == "precision" else L.FORM_PLAIN
    k, source = knobs(args)
    if w.preset == "reference":
        # The reference's constants; only the tree depth and the sort kernel
        # apply to its walk.
        k = {key: k[key] for key in ("lbits", "sort_variant")}
        source = {key: source[key] for key in k}
        return default_params(L.PRESET_REFERENCE, theta=args.theta, **k), source
    p = default_params(L.PRESET_PHYSICAL, theta=args.theta, form=form, **k, **w.physics)
    return p.replace(flags=walk_flags(args, L, p.flags)), source


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons; only the samples
    taken between mark_start() and mark_end() (the timed region) count."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.window = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.5)  # let the sampler start before the timed region
        except OSError:
            self.proc = None
        return self

    def mark_start(self):
        self._t0 = datetime.datetime.now()

    def mark_end(self):
        self.window = (self._t0, datetime.datetime.now())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        rows = []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f")
                rows.append((ts, float(f[2]), float(f[3]), f[6:10]))
            except ValueError:
                continue
        if not rows:
            return None
        inside = rows
        if self.window:
            lo, hi = self.window
            inside = [r for r in rows if lo <= r[0] <= hi] or rows
        reasons = {n for r in inside for n, v in zip(names, r[3]) if v.lower().startswith("active")}
        return {"sm_mhz": float(np.median([r[1] for r in inside])), "sm_max_mhz": inside[-1][2],
                "reasons": sorted(reasons), "samples": len(inside),
                "window": "samples inside the timed region" if inside is not rows
                          else "all samples (none fell inside the timed region)"}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text()), "measured"
    return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0}, "fallback"


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reduce_max(value: float, world: int) -> float:
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64,
                     device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def stage_bytes(n, key_bits, layer_counts, nsys, precision):
    """Algorithmic HBM bytes of each stage of one PHYSICAL step.

    bbox+encode: positions read twice (bbox, then encode) and the key written.
    sort+reorder: 8 B/key for the histogram read, 24 B/key per 8-bit pass
    (key and index read and written; 4 B less on the first pass, whose
    indices are generated), then the reorder reads the permutation and
    moves position, velocity and id (and the FP64 position).
    build: keys read once by the topology pass, which writes three 4-byte
    links per node (first particle, first child, parent); positions read
    once by the leaf pass; every node written
    once (key 8, sums 16/32, centre of mass 16, ranges 16, quadrupole 20,
    opening radius 4) and read once by its parent (sums, centre of mass,
    quadrupole, range: 68/84).
    integrate (kick-drift): position, velocity and acceleration read,
    position and velocity written (plus the FP64 position read and written).
    """
    passes = (key_bits + 7) // 8
    x64 = 24 if precision else 0
    nodes = int(sum(layer_counts))
    children = nodes - nsys
    s_node = 8 + (32 if precision else 16) + 16 + 16 + 20 + 4
    child_read = (32 if precision else 16) + 16 + 20 + 16
    return {
        "bbox+encode": (2 * (x64 or 16) + 8) * n,
        "sort+reorder": (8 + 24 * passes - 4) * n + (4 + 2 * (16 + 16 + 4 + x64)) * n,
        "build": (8 + 16 + x64) * n + nodes * (12 + s_node) + children * child_read,
        "integrate": (80 + 2 * x64) * n,
    }


def sort_alone(torch, n, key_bits, seed, flush, stream, sim, peaks):
    """astro_radix_sort of n uniform keys of key_bits, after an L2 flush each
    time: mean of three timed sorts and the HBM roofline figures."""
    from astro_gb300.radix_sort import RadixSort

    g = torch.Generator(device="cuda").manual_seed(seed)
    keys = torch.randint(0, 1 << 62, (n,), device="cuda", generator=g, dtype=torch.int64)
    if key_bits < 63:
        keys &= (1 << key_bits) - 1
    keys_out = torch.empty_like(keys)
    idx_out = torch.empty(n, dtype=torch.int32, device="cuda")
    sorter = RadixSort(n, key_bits)
    sort_ms = []
    for it in range(4):
        with torch.cuda.stream(stream):
            flush.fill_(3)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sorter.sort(keys, None, keys_out, idx_out, n, stream=sim.stream)
            e1.record(stream)
        sim.synchronize()
        if it:
            sort_ms.append(e0.elapsed_time(e1))
    sorter.status(sim.stream)
    passes = (key_bits + 7) // 8
    sort_b = (8 + 24 * passes - 4) * n
    ms = float(np.mean(sort_ms))
    return {"bound": "hbm", "key_bits": key_bits, "passes": passes, "keys": n, "bytes": sort_b,
            "ms": ms, "achieved": sort_b / (ms * 1e-3) / 1e9, "peak": peaks["hbm_gbs"],
            "unit": "GB/s", "frac": sort_b / (ms * 1e-3) / 1e9 / peaks["hbm_gbs"]}


def error_vs_direct(sim, n, seed, samples):
    """Median and p99 relative acceleration error against the FP64 direct
    sum on sampled particles (current state; forces only, the state is kept)."""
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(n, size=min(samples, n), replace=False)).astype(np.uint32)
    sim.generate_morton_codes()
    sim.sort()
    sim.build_tree()
    sim.barnes_hut()
    acc = sim.read_accel()
    direct = sim.direct_accel_f64(idx)
    sim.update_spheres(0.0)
    err = np.linalg.norm(acc[idx, :3] - direct, axis=1) / np.linalg.norm(direct, axis=1)
    return {"median": float(np.median(err)), "p99": float(np.percentile(err, 99)),
            "samples": int(len(err))}


def timed_steps(torch, sim, dt, steps, flush, stream):
    """K steps, each after an L2 flush, timed by CUDA events on the
    context's stream; returns the per-step milliseconds. A step whose group
    walk outgrew its buffers is evaluated again after the events (its timed
    run skipped the evaluation), so such a run is timed once more."""
    for _ in range(2):
        reruns = sim.walk_buffers()[2]
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        with torch.cuda.stream(stream):
            for k in range(steps):
                flush.fill_(k & 0xFF)
                starts[k].record(stream)
                sim.draw(dt, 1)
                ends[k].record(stream)
        sim.synchronize()
        torch.cuda.synchronize()
        if sim.walk_buffers()[2] == reruns:
            return [s.elapsed_time(e) for s, e in zip(starts, ends)]
    raise RuntimeError("the group walk outgrew its buffers during the timed steps twice")


# ---------------------------------------------------------------- ours --

def run_ours(args, world, rank, local):
    import torch

    import astro_gb300 as ag
    from astro_gb300 import layouts as L

    torch.cuda.set_device(local)
    w = workload(args)
    desc, dt = w.description, w.dt
    pm, vr, sizes = w.make()
    total_n = len(pm)
    sharded = bool(sizes) and world > 1
    if sharded:
        # The batching form shards by system: this rank steps its contiguous
        # range of systems (balanced by N log N), with no exchange.
        from astro_gb300 import shard

        if len(sizes) < world:
            raise SystemExit("fewer systems than ranks")
        rng = shard.partition_systems(sizes, world)[rank]
        a, b = shard.particle_range(sizes, rng)
        pm, vr, sizes = pm[a:b].copy(), vr[a:b].copy(), sizes[rng[0]:rng[1]]
    n = len(pm)
    # Particles all ranks advance per step: replicas each step a whole copy.
    job_n = total_n if sharded else n * world
    form = L.FORM_PRECISION if args.form == "precision" else L.FORM_PLAIN
    p, knob_source = make_params(args, L, ag.default_params)
    nsys = len(sizes) if sizes else 1
    is_ref = w.preset == "reference"
    ct, n_tree = w.make_colors() if is_ref else (None, n)
    sim = ag.Simulation(p, max_n=n, max_systems=nsys)

    def upload_from(pm_, vr_):
        if sizes:
            sim.upload_systems(pm_, vr_, sizes)
        else:
            sim.upload(pm_, vr_, ct, n_tree=n_tree)

    upload_from(pm, vr)
    stream = torch.cuda.ExternalStream(sim.stream)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    # Warm-up (also captures the step graph).
    for _ in range(args.warmup):
        sim.draw(dt, 1)
    sim.synchronize()

    # Timed region: K steps, each after an L2 flush, timed by CUDA events on
    # the context's stream.
    barrier(world)
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        clk.mark_start()
        t0 = time.perf_counter()
        step_ms = timed_steps(torch, sim, dt, args.steps, flush, stream)
        wall = time.perf_counter() - t0
        clk.mark_end()
    barrier(world)
    t_ms = sum(step_ms)
    t_ms_max = reduce_max(t_ms, world)
    value = job_n * args.steps / (t_ms_max * 1e-3)

    # One instrumented step: per-stage times.
    stages = {}
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
    with torch.cuda.stream(stream):
        flush.fill_(1)
        ev[0].record(stream)
        sim.generate_morton_codes()
        ev[1].record(stream)
        sim.sort()
        ev[2].record(stream)
        sim.build_tree()
        ev[3].record(stream)
        sim.barnes_hut()
        ev[4].record(stream)
        sim.update_spheres(dt)
        ev[5].record(stream)
    sim.synchronize()
    for i, name in enumerate(["bbox+encode", "sort+reorder", "build", "traverse", "integrate"]):
        stages[name] = ev[i].elapsed_time(ev[i + 1])
    interactions, visits, cell_inter = sim.read_stats(cells=True)
    sizes_, offsets, counts = sim.tree_info()
    peaks, peak_src = measured_peaks()
    key_bits = 3 * p.lbits + ((nsys - 1).bit_length() if nsys > 1 else 0)
    stage_roofline = None
    if not is_ref:
        sbytes = stage_bytes(n, key_bits, counts, nsys, form == L.FORM_PRECISION)
        stage_roofline = {
            k: {"bytes": int(b), "ms": stages[k], "achieved_gbs": b / (stages[k] * 1e-3) / 1e9,
                "frac": b / (stages[k] * 1e-3) / 1e9 / peaks["hbm_gbs"]}
            for k, b in sbytes.items()}

    # The pair sort alone (astro_radix_sort) on uniform keys of the step's
    # width and length, after an L2 flush: the sort stage's HBM roofline
    # (PHYSICAL workloads; the reference's scene sorts only its 205 tree bodies).
    sort_roofline = None
    if not is_ref:
        sort_roofline = sort_alone(torch, n, key_bits, w.seed, flush, stream, sim, peaks)
    quad = (p.flags & L.FLAG_QUADRUPOLE) != 0
    group = not is_ref and args.walk == "group"

    far_nodes, far_inter = sim.read_far_stats() if not is_ref else (0, 0)
    flops = (FLOPS_PER_QUAD_CELL if quad else FLOPS_PER_INTERACTION) * (cell_inter - far_inter) + \
        FLOPS_PER_INTERACTION * (interactions - cell_inter) + FLOPS_PER_FAR_NODE * far_nodes + \
        (FLOPS_PER_FAR_EVAL * n if far_nodes else 0)

    # Traversal alone, several launches after a flush each, for the roofline:
    # the group walk timed apart from its evaluation (the far-node sums
    # and the evaluation kernel; events recorded by the library between
    # them), the other walks as one kernel.
    trav_ms, walk_ms, eval_ms = [], [], []
    for _ in range(3):
        with torch.cuda.stream(stream):
            sim.generate_morton_codes()
            sim.sort()
            sim.build_tree()
            flush.fill_(2)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sim.barnes_hut()
            e1.record(stream)
            sim.update_spheres(0.0)
        sim.synchronize()
        trav_ms.append(e0.elapsed_time(e1))
        if group:
            wm, em = sim.traverse_times()
            walk_ms.append(wm)
            eval_ms.append(em)
    trav = float(np.mean(trav_ms))
    kernel_ms = float(np.mean(eval_ms)) if group else trav
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    fp32_peak = 2 * 128 * sms * peaks.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
    achieved = flops / (kernel_ms * 1e-3) / 1e12

    # Error against the FP64 direct sum on sampled particles (PHYSICAL units only).
    err = None if is_ref else error_vs_direct(sim, n, w.seed, args.error_samples)

    # End to end through the C ABI with pinned host buffers: every step
    # uploads its input particles and downloads its result. The transfers
    # are pipelined (astro_upload_async / astro_download_async): the next
    # step's upload and the last step's download run on their own copy
    # streams while a step computes.
    e2e = None
    if not args.no_e2e:
        def pinned(dtype):
            buf = torch.empty(n * 32, dtype=torch.uint8, pin_memory=True)
            return buf, buf.numpy().view(dtype)

        (b_pm, hpm), (b_vr, hvr) = pinned(L.POSITION_MASS), pinned(L.VELOCITY_RADIUS)
        (b_opm, opm), (b_ovr, ovr) = pinned(L.POSITION_MASS), pinned(L.VELOCITY_RADIUS)
        hpm[:] = pm
        hvr[:] = vr
        upload_from(hpm, hvr)

        def e2e_steps(k):
            for _ in range(k):
                sim.upload_async(hpm, hvr)
                sim.draw(dt, 1)
                sim.download_async(opm, ovr)
            sim.synchronize()

        e2e_steps(max(1, args.warmup))
        barrier(world)
        t0 = time.perf_counter()
        e2e_steps(args.steps)
        te = time.perf_counter() - t0
        te = reduce_max(te, world)
        e2e = {"value": job_n * args.steps / te, "unit": UNIT,
               "h2d_bytes_per_step": 64 * n, "d2h_bytes_per_step": 64 * n,
               "ms_per_step": te * 1e3 / args.steps,
               "how": "pinned host buffers; per step astro_upload_async, astro_step, "
                      "astro_download_async (copies overlap the steps), one synchronize at the end"}

    launches_per_step = kernels_per_step(key_bits, sizes_, w.preset)
    sim.close()
    del flush
    torch.cuda.empty_cache()
    return dict(n=n, sharded=sharded, desc=desc, dt=dt, p=p, knob_source=knob_source, value=value,
                t_ms=t_ms_max,
                wall=wall, step_ms=step_ms, stages=stages, interactions=interactions,
                visits=visits, cell_inter=cell_inter, flops=flops, far_nodes=far_nodes,
                far_inter=far_inter, counts=[int(c) for c in counts], trav_ms=trav,
                kernel_ms=kernel_ms, walk_ms=float(np.mean(walk_ms)) if walk_ms else None,
                achieved=achieved, fp32_peak=fp32_peak, peak_src=peak_src, err=err, e2e=e2e,
                clocks=clk.summary(), launches=launches_per_step * args.steps, sizes=sizes, pm=pm,
                vr=vr, stage_roofline=stage_roofline, sort_roofline=sort_roofline)


def run_variant(torch, args, workload_name, form, lbits, steps, warmup, error_samples=512,
                theta=None):
    """Another configuration of the line: workload `workload_name` in `form`
    at tree depth `lbits` (None: tuned), its tuned knobs, opening angle
    `theta` (None: the line's), `steps` timed steps after an L2 flush each.
    Returns its throughput, step time, knobs and error (PHYSICAL workloads)."""
    import astro_gb300 as ag
    from astro_gb300 import layouts as L

    va = argparse.Namespace(**{**vars(args), "workload": workload_name, "form": form,
                               "lbits": lbits, "n": None, "bucket": None, "warps": None,
                               "group_size": None, "sort_variant": None, "delta_weight": None,
                               "far_ratio": None, "walk_frontier": None,
                               "theta": args.theta if theta is None else theta})
    w = WORKLOADS[workload_name]
    pm, vr, sizes = w.make()
    n = len(pm)
    p, source = make_params(va, L, ag.default_params)
    sim = ag.Simulation(p, max_n=n, max_systems=len(sizes) if sizes else 1)
    try:
        if sizes:
            sim.upload_systems(pm, vr, sizes)
        else:
            sim.upload(pm, vr)
        stream = torch.cuda.ExternalStream(sim.stream)
        flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
        for _ in range(warmup):
            sim.draw(w.dt, 1)
        sim.synchronize()
        ms = timed_steps(torch, sim, w.dt, steps, flush, stream)
        err = error_vs_direct(sim, n, w.seed, error_samples)
        k, _ = knobs(va)
        return {"workload": f"{workload_name}: {w.description}", "form": form, "lbits": p.lbits,
                "theta": p.theta,
                "value": n * steps / (sum(ms) * 1e-3), "unit": UNIT,
                "ms_per_step": float(np.mean(ms)), "steps": steps, "knobs": k,
                "knob_source": source, "error_vs_fp64_direct": err}
    finally:
        sim.close()
        torch.cuda.empty_cache()


def one_at_a_time(torch, args, steps, warmup):
    """The batching workload's systems stepped one at a time in plain FP32:
    one context and step graph per system, each system's step launched
    after the previous one finished (an event chain across the contexts'
    streams, no host synchronisation)."""
    import astro_gb300 as ag
    from astro_gb300 import layouts as L

    w = WORKLOADS["c4"]
    pm, vr, sizes = w.make()
    va = argparse.Namespace(**{**vars(args), "workload": "c4", "form": "plain", "lbits": None,
                               "n": None})
    p, _ = make_params(va, L, ag.default_params)
    sims, off = [], 0
    try:
        for sz in sizes:
            s1 = ag.Simulation(p, max_n=sz)
            s1.upload(pm[off:off + sz], vr[off:off + sz])
            off += sz
            s1.draw(w.dt, max(1, warmup))
            sims.append(s1)
        for s1 in sims:
            s1.synchronize()
        streams = [torch.cuda.ExternalStream(s1.stream) for s1 in sims]
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(streams[0])
        prev = e0
        for _ in range(steps):
            for s1, st1 in zip(sims, streams):
                st1.wait_event(prev)
                s1.draw(w.dt, 1)
                prev = torch.cuda.Event()
                prev.record(st1)
        streams[0].wait_event(prev)
        e1.record(streams[0])
        torch.cuda.synchronize()
        t1 = e0.elapsed_time(e1)
        return {"value": len(pm) * steps / (t1 * 1e-3), "unit": UNIT, "steps": steps,
                "ms_per_step": t1 / steps, "form": "plain",
                "how": "plain FP32, one context and step graph per system, each system's step "
                       "waiting for the previous one"}
    finally:
        for s1 in sims:
            s1.close()
        torch.cuda.empty_cache()


def extras(args):
    """The default line's other configurations: C5 at lbits 21 (63-bit keys),
    in the precision form and at opening angles 0.3, 0.5 and 1.0, and the
    batching workload plain batched, precision + batched and one system at
    a time."""
    import torch

    k = max(3, args.steps // 4)
    out = {}
    if args.workload == "c5" and args.form == "plain":
        out["c5_lbits21"] = run_variant(torch, args, "c5", "plain", 21, k, args.warmup)
        out["c5_precision"] = run_variant(torch, args, "c5", "precision", 6, k, args.warmup)
        # The configuration's opening-angle sweep at lbits 6, the line's knobs.
        out["c5_theta_sweep"] = [run_variant(torch, args, "c5", "plain", 6, 3, 1, theta=t)
                                 for t in (0.3, 0.5, 1.0)]
    plain = run_variant(torch, args, "c4", "plain", None, k, args.warmup)
    prec = run_variant(torch, args, "c4", "precision", None, k, args.warmup)
    alone = one_at_a_time(torch, args, max(2, k // 2), args.warmup)
    out["batching"] = {
        "workload": plain["workload"], "plain_batched": plain, "precision_batched": prec,
        "plain_one_at_a_time": alone,
        "precision_batched_over_plain_batched": prec["value"] / plain["value"],
        "precision_batched_over_one_at_a_time": prec["value"] / alone["value"]}
    return out


# ----------------------------------------------------------- CPU side --

def cpu_step(orc, w, p, pm_c, vr_c, sizes, dt):
    """One step of the CPU restatement in place (64 one-bit split passes per
    sort, as the reference)."""
    if w.preset == "reference":
        ct, n_tree = w.make_colors()
        orc.ref_run(p, pm_c, vr_c, ct, n_tree=n_tree, dt=dt, steps=1, split_passes=64)
    else:
        orc.phys_run(p, pm_c, vr_c, sizes=sizes, dt=dt, steps=1, split_passes=64)


def cpu_run(args, pm, vr, sizes, p, dt, budget_s):
    """The CPU restatement on all host cores: whole steps of the same
    workload until the time budget is spent (at least one)."""
    from oracle import oracle as orc

    cores = orc.set_threads(args.cpu_threads)
    steps, t_total = 0, 0.0
    pm_c, vr_c = pm.copy(), vr.copy()
    w = workload(args)
    while True:
        t0 = time.perf_counter()
        cpu_step(orc, w, p, pm_c, vr_c, sizes, dt)
        t_total += time.perf_counter() - t0
        steps += 1
        if t_total >= budget_s:
            break
    return {"value": len(pm) * steps / t_total, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{steps} whole step(s) of the same workload (N={len(pm)}), 64 one-bit "
                      f"split passes per sort, {t_total:.1f} s"}


def run_reference(args):
    """--impl reference: the CPU restatement timed on the host cores. Inputs
    and parameters are made without loading the CUDA library (the
    generators come from the oracle's build of the same host source)."""
    from astro_gb300 import ic
    from astro_gb300 import layouts as L
    from oracle import oracle as orc

    ic.use_generator_library(orc.lib())
    w = workload(args)
    desc, dt = w.description, w.dt
    pm, vr, sizes = w.make()
    n = len(pm)
    form = L.FORM_PRECISION if args.form == "precision" else L.FORM_PLAIN
    p, knob_source = make_params(args, L, L.host_default_params)
    cores = orc.set_threads(args.cpu_threads)
    pm_c, vr_c = pm.copy(), vr.copy()
    # Warm-up: at most one step (a CPU step warms nothing up beyond the first).
    for _ in range(min(args.warmup, 1)):
        cpu_step(orc, w, p, pm_c, vr_c, sizes, dt)
    # Timed: up to K whole steps, stopping once the time budget is spent.
    steps, t = 0, 0.0
    while steps < max(1, args.steps):
        t0 = time.perf_counter()
        cpu_step(orc, w, p, pm_c, vr_c, sizes, dt)
        t += time.perf_counter() - t0
        steps += 1
        if t >= args.reference_seconds:
            break
    value = n * steps / t
    sample = (f"{steps} whole step(s) of the workload (N={n}) of the {args.steps} asked, within a "
              f"{args.reference_seconds:g} s budget; 64 one-bit split passes per sort")
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "steps": steps,
        "warmup": min(args.warmup, 1), "ms_per_step": t * 1e3 / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32" if form == 0 else "f32+f64",
        "data": "synthetic (seeded, Philox4x32-10)", "impl": "reference",
        "config": config_dict(args, desc, n, dt, p, knob_source),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def config_dict(args, desc, n, dt, p, knob_source, shards=1):
    walk = ("per-particle (the reference's)" if p.preset == 0
            else "per-particle" if p.flags & 0x20 else "group")
    return {"workload": f"{args.workload}: {desc}", "n": n,
            "preset": "PHYSICAL" if p.preset == 1 else "REFERENCE",
            "form": args.form, "walk": walk, "quadrupole": bool(p.flags & 0x10),
            "opening": (f"size/theta + {p.open_delta_weight:g} delta" if p.flags & 0x8
                        else "size/theta"),
            "theta": p.theta, "eps": p.softening, "dt": dt, "G": p.g,
            "lbits": p.lbits, "key_bits": 3 * p.lbits, "layers": p.lbits + 1,
            "bucket": p.bucket, "group_size": p.group_size or 32,
            "block_warps": p.block_warps or 4, "sort_variant": p.sort_variant,
            "open_delta_weight": p.open_delta_weight, "far_ratio": p.far_ratio,
            "walk_frontier": p.walk_frontier,
            "knob_source": knob_source,
            "l2": "flushed (256 MB write) before every timed step",
            "parallelism": (f"systems sharded over {shards} GPUs (contiguous ranges balanced by "
                            "N log N, no exchange; n is rank 0's share)" if shards > 1
                            else "replicas (one independent system per GPU)")}


def main(argv=None):
    args = parse(argv)
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(run_reference(args)))
        return 0
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    r = run_ours(args, world, rank, local)
    if rank == 0:
        extra = None
        if not args.no_extras and args.n is None and args.workload in ("c5", "c4"):
            extra = extras(args)
        cpu = None
        if not args.no_cpu:
            cpu = cpu_run(args, r["pm"], r["vr"], r["sizes"], r["p"], r["dt"], args.cpu_seconds)
        group = WORKLOADS[args.workload].preset != "reference" and args.walk == "group"
        line = {
            "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": r["t_ms"] / args.steps, "higher_is_better": True,
            "scaling": "strong" if r["sharded"] else "weak",
            "vs_baseline": None, "dtype": "f32" if args.form == "plain" else "f32+f64",
            "data": "synthetic (seeded, Philox4x32-10)",
            "config": config_dict(args, r["desc"], r["n"], r["dt"], r["p"], r["knob_source"],
                                  world if r["sharded"] else 1),
            "e2e": r["e2e"], "gpu_launches": r["launches"],
            "roofline": {"kernel": ("traverse_ref_kernel"
                                    if WORKLOADS[args.workload].preset == "reference"
                                    else ("group_far_kernel + group_eval_kernel"
                                          if r["far_nodes"] and r["p"].group_size > 32
                                          else "group_eval_kernel") if group
                                    else "traverse_phys_kernel"),
                         "bound": "fp32",
                         "achieved": r["achieved"], "peak": r["fp32_peak"], "unit": "TFLOP/s",
                         "frac": r["achieved"] / r["fp32_peak"],
                         "traffic": NCU_EVAL_DRAM_BYTES.get((args.workload, args.form,
                                                             r["p"].lbits)),
                         "flops_per_launch": r["flops"],
                         "interactions_per_s": r["interactions"] / (r["kernel_ms"] * 1e-3),
                         "launch_ms": r["kernel_ms"],
                         "walk_kernel_ms": r["walk_ms"], "traversal_ms": r["trav_ms"],
                         "peak_source": f"2 x 128 FP32 lanes x SMs x sm_max_mhz ({r['peak_src']} peaks file)"},
            "cpu_baseline": cpu, "clocks": r["clocks"],
            "error_vs_fp64_direct": r["err"],
            "interactions_per_particle": r["interactions"] / r["n"],
            "cell_interactions_per_particle": r["cell_inter"] / r["n"],
            "far_interactions_per_particle": r["far_inter"] / r["n"],
            "far_nodes": r["far_nodes"],
            "node_visits_per_particle": r["visits"] / r["n"],
            "stages_ms": r["stages"], "stage_roofline_hbm": r["stage_roofline"],
            "sort_roofline": r["sort_roofline"], "layer_counts": r["counts"],
        }
        if extra:
            line["extras"] = extra
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
