"""Host-side logic without a GPU: workload definitions, the autotuner's
search space and result file, and the benchmark's knob resolution."""
import json
import sys
from pathlib import Path
from types import SimpleNamespace

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_workloads_match_their_descriptions():
    from astro_gb300.workloads import WORKLOADS

    assert sorted(WORKLOADS) == ["c1", "c2", "c3", "c4", "c5", "ref"]
    assert WORKLOADS["ref"].preset == "reference" and WORKLOADS["ref"].lbits == 6
    assert WORKLOADS["c2"].n == 524288 and WORKLOADS["c5"].n == 1 << 24
    assert WORKLOADS["c4"].generator == "batch"
    assert len({w.seed for w in WORKLOADS.values()}) == 6


def test_autotune_candidates_stay_in_range():
    from astro_gb300 import autotune

    for n in (16, 16384, 524288, 1 << 22, 1 << 24):
        c = autotune.candidates("lbits", n)
        assert c == sorted(c) and all(3 <= v <= 21 for v in c)
    assert autotune.candidates("group_size", 1000)[-1] == 64  # two particles per lane
    assert set(autotune.candidates("block_warps", 1)) <= {2, 4, 8}
    assert autotune.candidates("sort_variant", 1) == list(range(1, 13))
    assert all(0 < w < 1 for w in autotune.candidates("open_delta_weight", 1))
    assert all(0 < r <= 0.5 for r in autotune.candidates("far_ratio", 1))
    assert set(autotune.ACCURACY_KNOBS) <= set(autotune.KNOBS)
    with pytest.raises(KeyError):
        autotune.candidates("theta", 1)


def test_tuned_file_feeds_bench_knobs(tmp_path, monkeypatch):
    from astro_gb300 import autotune

    f = tmp_path / "tuned.json"
    f.write_text(json.dumps({"results": {"c2/plain": {"knobs": {
        "lbits": 12, "bucket": 32, "group_size": 16, "block_warps": 8, "sort_variant": 3}}}}))
    monkeypatch.setattr(autotune, "TUNED_PATH", f)
    sys.path.insert(0, str(ROOT))
    import bench

    args = SimpleNamespace(workload="c2", form="plain", no_tuned=False, lbits=None, bucket=20,
                           warps=None, group_size=None, sort_variant=None, delta_weight=None,
                           far_ratio=None, walk_frontier=None)
    k, src = bench.knobs(args)
    assert k == {"lbits": 12, "bucket": 20, "block_warps": 8, "group_size": 16, "sort_variant": 3,
                 "open_delta_weight": 1.0, "far_ratio": 0.0, "walk_frontier": 0}
    assert src["bucket"] == "command line" and src["lbits"] == "autotuner"
    args.form = "precision"  # no entry: preset defaults
    k, src = bench.knobs(args)
    assert k["lbits"] == 14 and k["group_size"] == 0 and src["lbits"] == "default"
    args.form, args.no_tuned = "plain", True
    assert bench.knobs(args)[0]["lbits"] == 14


def test_autotune_load_without_file(tmp_path, monkeypatch):
    from astro_gb300 import autotune

    monkeypatch.setattr(autotune, "TUNED_PATH", tmp_path / "absent.json")
    assert autotune.load() == {}


def test_driver_arguments():
    from astro_gb300 import driver

    a = driver.parse(["--scene", "plummer", "--n", "100", "--steps", "7", "--save-every", "3"])
    assert (a.scene, a.n, a.steps, a.save_every, a.resume) == ("plummer", 100, 7, 3, None)
    assert set(driver.SCENES) >= {"reference", "disk_bulge", "uniform_cube"}


def test_bench_reference_arm_prints_the_contract_line():
    # The reference arm (CPU restatement) on the small workload: one JSON
    # line with the metric, the impl tag, the CPU baseline and a zero-copy e2e.
    import subprocess

    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                          "--workload", "c1", "--steps", "1", "--warmup", "0", "--cpu-threads", "2"],
                         capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "particle-updates/s"
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] == 2
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert line["config"]["workload"].startswith("c1") and line["config"]["n"] == 16384


def test_bench_kernel_count_per_step():
    # The launch list of one c2 step before the climbing build: 3 (bbox,
    # setup, encode) + histogram + 5 passes + reorder + topology + 13
    # aggregations + traversal = 25; the climb folds the layers under 32,768
    # nodes into one launch.
    sys.path.insert(0, str(ROOT))
    import bench

    c2_layers = [524288] * 6 + [262144, 32768, 4096, 512, 64, 8, 1]
    # PHYSICAL: the group walk and its evaluation are two launches.
    assert bench.kernels_per_step(36, c2_layers) == 9 + 5 + 8
    assert bench.kernels_per_step(18, [205] * 7, "reference") == 8 + 3
    assert bench.kernels_per_step(21, [2 ** 21, 2 ** 18, 2 ** 15, 4096, 512, 64, 8, 1]) == 9 + 3 + 3


def test_bench_quotes_c5_at_the_reference_depth(tmp_path, monkeypatch):
    # The default line is C5 at lbits 6 (the reference's 7 layers), taking
    # the knobs the autotuner found at that depth.
    from astro_gb300 import autotune

    f = tmp_path / "tuned.json"
    f.write_text(json.dumps({"results": {
        "c5/plain": {"knobs": {"lbits": 7, "group_size": 32}},
        "c5/plain@lbits6": {"knobs": {"lbits": 6, "group_size": 64, "far_ratio": 0.4}}}}))
    monkeypatch.setattr(autotune, "TUNED_PATH", f)
    sys.path.insert(0, str(ROOT))
    import bench

    args = bench.parse([])
    assert args.workload == "c5" and args.form == "plain"
    k, src = bench.knobs(args)
    assert k["lbits"] == 6 and k["group_size"] == 64 and k["far_ratio"] == 0.4
    assert src["lbits"] == "the workload's quoted depth" and src["group_size"] == "autotuner"
    args = bench.parse(["--lbits", "21"])  # no entry at 21: the workload's entry, lbits given
    k, src = bench.knobs(args)
    assert k["lbits"] == 21 and k["group_size"] == 32 and src["lbits"] == "command line"


def test_host_defaults_and_generators_match_the_library(native):
    """The reference arm builds parameters and particles without the CUDA
    library: its host restatement of astro_params_default and the oracle's
    build of the generators must give the library's bytes."""
    import ctypes

    import numpy as np

    from astro_gb300 import ic, layouts as L
    from astro_gb300.simulation import default_params
    from oracle import oracle as orc

    for preset in (L.PRESET_REFERENCE, L.PRESET_PHYSICAL):
        a, b = default_params(preset), L.host_default_params(preset)
        assert ctypes.string_at(ctypes.addressof(a), ctypes.sizeof(a)) == \
            ctypes.string_at(ctypes.addressof(b), ctypes.sizeof(b))
    made = {}
    for gen in (None, orc.lib()):
        ic.use_generator_library(gen)
        try:
            made[gen is None] = [ic.plummer(1000, 3), ic.disk_bulge(1000, 4),
                                 ic.two_plummer(1000, 5), ic.uniform_cube(1000, 6),
                                 ic.reference_scene(5, 20, 100, seed=7), ic.system_sizes(7, 8)]
        finally:
            ic.use_generator_library(None)
    for x, y in zip(made[True], made[False]):
        for u, v in zip(x, y):
            assert np.array_equal(u, v)


def test_reference_arm_does_not_load_the_cuda_library():
    """bench.py --impl reference runs the CPU restatement only: the process
    never maps libastro_cuda.so."""
    import subprocess

    code = ("import sys, json; sys.path.insert(0, %r); import bench; "
            "line = bench.run_reference(bench.parse(['--impl', 'reference', '--workload', 'c1', "
            "'--steps', '1', '--warmup', '0', '--cpu-threads', '2'])); "
            "maps = open('/proc/self/maps').read(); "
            "print(json.dumps({'cuda_lib': 'libastro_cuda' in maps, "
            "'oracle': 'liboracle_astro' in maps}))" % str(ROOT))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300,
                         cwd=ROOT)
    assert out.returncode == 0, out.stderr
    res = json.loads(out.stdout.strip().splitlines()[-1])
    assert res == {"cuda_lib": False, "oracle": True}
