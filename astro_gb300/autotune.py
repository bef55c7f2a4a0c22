"""Autotuner of the Barnes-Hut step's launch knobs on the current GPU.

The search runs in the library (astro_autotune / astro_autotune_ex,
astro_gb300/csrc/tune.cu) on a context's own particles; this module drives
it over the benchmark workloads and collects the results file.

The knobs are fields of astro_params that change speed, not physics:

  block_warps   traversal block size (warps per block: 4 or 8)
  group_size    particles per warp: consecutive sorted particles sharing one
                tree walk (1..64; two per lane above 32; groups of <= 16 run
                as several copies that split the source lists)
  lbits         tree depth, i.e. the depth of the walk (layers = lbits + 1)
  bucket        leaf tile size: an opened node holding <= bucket particles
                is summed particle by particle
  sort_variant  radix sort pass kernel (items per thread / blocks per SM /
                ranking / pipelined / lean)
  walk_frontier the group walk's frontier: runs of consecutive child nodes
                or a list of node indices

  far_ratio     accepted nodes further than (group radius) / far_ratio from
                the group's centre are summed through one second-order
                expansion per group instead of per particle: larger ratios
                expand more nodes and cost accuracy
  open_delta_weight
                w of the opening radius size/theta + w |com - cell centre|:
                lower w opens fewer nodes and costs accuracy
far_ratio and open_delta_weight are only moved while the error stays within
0.8 x the target (or within 2% of the starting error where theta alone puts
that above 0.8 x the target).

theta, the softening, the quadrupole and opening-radius flags and the form
(plain / precision) are physics and stay as given.

Search: coordinate descent from the preset's defaults over the speed knobs,
then every (open_delta_weight, far_ratio) pair (far_ratio rising until the
error leaves its bound), then lbits, bucket, group_size, block_warps and
walk_frontier once more. Each knob in turn is swept with the others fixed; the fastest setting
is kept among those whose
median relative acceleration error against the FP64 direct sum (on sampled
particles) is at most max(target, 1.02 x the starting error) (max(0.8 x the
target, 1.02 x the starting error) for the accuracy knobs). A step's time is
the CUDA-event time of graph-replayed steps (dt = 0, so every trial sees the
same particles); the sort variant is judged by the sort stage's own time.

  python -m astro_gb300.autotune --workloads c1,c2,c3,c4,c5 --forms plain,precision \\
      [--lbits L] [--from-tuned] [--out astro_gb300/tuned.json]

The result file holds, per "workload/form", the chosen knobs, the step time
and error they gave, and every trial; bench.py reads it for its defaults.
"""
from __future__ import annotations

import argparse
import datetime
import json
import sys
from pathlib import Path

import numpy as np

from . import layouts as L
from .simulation import Simulation, default_params
from .workloads import WORKLOADS

TUNED_PATH = Path(__file__).resolve().parent / "tuned.json"
KNOBS = ("lbits", "bucket", "group_size", "block_warps", "sort_variant", "walk_frontier",
         "far_ratio", "open_delta_weight")
ACCURACY_KNOBS = ("far_ratio", "open_delta_weight")
FORMS = {"plain": L.FORM_PLAIN, "precision": L.FORM_PRECISION}


def candidates(knob: str, n: int) -> list[int]:
    """The values the library's search tries for a knob (n: the largest
    system's particle count)."""
    if knob == "lbits":
        # From about 8 particles per finest cell down to single occupancy.
        lo = max(3, int(np.ceil(np.log2(max(n, 8) / 8) / 3)))
        return sorted({min(21, v) for v in (lo, lo + 1, lo + 2, lo + 4, lo + 6)})
    if knob == "bucket":
        return [8, 16, 32, 64]
    if knob == "group_size":
        return [8, 12, 16, 24, 32, 48, 64]
    if knob == "block_warps":
        return [4, 8]
    if knob == "sort_variant":
        return list(range(1, 13))
    if knob == "walk_frontier":
        return [0, 1]
    if knob == "far_ratio":
        return [0.1, 0.15, 0.2, 0.25, 0.3, 0.4, 0.5]
    if knob == "open_delta_weight":
        return [0.85, 0.7, 0.5]
    raise KeyError(knob)


def result_key(workload: str, form: str, lbits: int | None = None) -> str:
    """Key of a result in the tuned file: "c2/plain", or "c5/plain@lbits6"
    for a search at a fixed tree depth."""
    return f"{workload}/{form}" + (f"@lbits{lbits}" if lbits is not None else "")


def tune(workload: str, form: str, target: float = 1e-3, samples: int = 1024,
         lbits: int | None = None, start: dict | None = None, log=print) -> dict:
    """Tune one workload with the library's native search
    (astro_autotune_keep) from the preset's defaults (or the knobs `start`)
    at the workload's starting depth, or holding the depth at `lbits`."""
    w = WORKLOADS[workload]
    pm, vr, sizes = w.make()
    knobs = dict(start or {})
    knobs["lbits"] = lbits if lbits is not None else knobs.get("lbits", w.lbits)
    params = default_params(L.PRESET_PHYSICAL, form=FORMS[form], **knobs, **w.physics)
    sim = Simulation(params, max_n=len(pm), max_systems=len(sizes) if sizes else 1)
    try:
        if sizes:
            sim.upload_systems(pm, vr, sizes)
        else:
            sim.upload(pm, vr)
        res = sim.autotune(target=target, samples=samples,
                           keep=L.TUNE_KEEP_LBITS if lbits is not None else 0)
    finally:
        sim.close()
    start = res["trials"][0]
    log(f"{workload}/{form} start {start['knobs']}: {start['ms']:.3f} ms, error "
        f"{start['median_error']:.3g}")
    best = start
    for t in res["trials"][1:]:
        if t["knobs"] == res["knobs"] and t["ms"] == res["ms"]:
            best = t
        log(f"  {t['knobs']}: {t['ms']:.3f} ms (sort {t['sort_ms']:.3f}), error "
            f"{t['median_error']:.3g}{'  <- chosen' if t is best else ''}")
    return {"workload": workload, "form": form, **res}


def load(path: Path | None = None) -> dict:
    """The tuned knobs per "workload/form" ({} when the file is absent)."""
    path = path or TUNED_PATH
    if not path.exists():
        return {}
    return json.loads(path.read_text()).get("results", {})


def main(argv=None) -> int:
    import torch

    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--workloads", default="c1,c2,c3,c4,c5")
    ap.add_argument("--forms", default="plain,precision")
    ap.add_argument("--target", type=float, default=1e-3)
    ap.add_argument("--lbits", type=int, default=None,
                    help="hold the tree depth (result key workload/form@lbitsL)")
    ap.add_argument("--from-tuned", action="store_true",
                    help="start each search from the knobs already in the file")
    ap.add_argument("--out", type=Path, default=TUNED_PATH)
    args = ap.parse_args(argv)
    prev = json.loads(args.out.read_text()) if args.out.exists() else {"results": {}}
    results = prev.get("results", {})
    for wl in args.workloads.split(","):
        for form in args.forms.split(","):
            key = result_key(wl, form, args.lbits)
            start = results.get(key, {}).get("knobs") if args.from_tuned else None
            r = tune(wl, form, args.target, lbits=args.lbits, start=start)
            results[key] = r
            out = {"device": torch.cuda.get_device_name(),
                   "sms": torch.cuda.get_device_properties(0).multi_processor_count,
                   "when": datetime.datetime.now(datetime.timezone.utc).isoformat(timespec="seconds"),
                   "method": "astro_autotune_ex: coordinate descent over " + ", ".join(KNOBS) +
                             "; step time by CUDA events over graph-replayed steps (dt = 0)",
                   "results": results}
            args.out.write_text(json.dumps(out, indent=1) + "\n")
    return 0


if __name__ == "__main__":
    sys.exit(main())
