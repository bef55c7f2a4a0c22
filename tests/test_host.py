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
    assert autotune.candidates("group_size", 1000)[-1] == 32
    assert set(autotune.candidates("block_warps", 1)) <= {2, 4, 8}
    assert autotune.candidates("sort_variant", 1) == list(range(1, 10))
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
    assert bench.kernels_per_step(36, c2_layers) == 8 + 5 + 8
    assert bench.kernels_per_step(18, [205] * 7) == 8 + 3
    assert bench.kernels_per_step(21, [2 ** 21, 2 ** 18, 2 ** 15, 4096, 512, 64, 8, 1]) == 8 + 3 + 3
