"""Autotuner of the Barnes-Hut step's launch knobs on the current GPU.

The knobs are fields of astro_params that change speed, not physics:

  block_warps   traversal block size (warps per block: 4 or 8)
  group_size    particles per warp: consecutive sorted particles sharing one
                tree walk (1..32; groups of <= 16 run as several copies that
                split the source lists)
  lbits         tree depth, i.e. the depth of the walk (layers = lbits + 1)
  bucket        leaf tile size: an opened node holding <= bucket particles
                is summed particle by particle
  sort_variant  radix sort pass kernel (items per thread / blocks per SM /
                ranking / pipelined)

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
error leaves its bound), then lbits, bucket, group_size and block_warps once
more. Each knob in turn is swept with the others fixed; the fastest setting
is kept among those whose
median relative acceleration error against the FP64 direct sum (on sampled
particles) is at most max(target, 1.02 x the starting error) (max(0.8 x the
target, 1.02 x the starting error) for the accuracy knobs). A step's time is
the CUDA-event time of graph-replayed steps (dt = 0, so every trial sees the
same particles); the sort variant is judged by the sort stage's own time.

  python -m astro_gb300.autotune --workloads c1,c2,c3,c4,c5 --forms plain,precision \\
      [--out astro_gb300/tuned.json]

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
KNOBS = ("lbits", "bucket", "group_size", "block_warps", "sort_variant", "far_ratio",
         "open_delta_weight")
ACCURACY_KNOBS = ("far_ratio", "open_delta_weight")
FORMS = {"plain": L.FORM_PLAIN, "precision": L.FORM_PRECISION}


def candidates(knob: str, n: int) -> list[int]:
    if knob == "lbits":
        # From about 8 particles per finest cell down to single occupancy.
        lo = max(3, int(np.ceil(np.log2(max(n, 8) / 8) / 3)))
        return sorted({min(21, v) for v in (lo, lo + 1, lo + 2, lo + 4, lo + 6)})
    if knob == "bucket":
        return [8, 16, 32, 64]
    if knob == "group_size":
        return [8, 12, 16, 24, 32]
    if knob == "block_warps":
        return [4, 8]
    if knob == "sort_variant":
        return list(range(1, 10))
    if knob == "far_ratio":
        return [0.1, 0.15, 0.2, 0.25, 0.3, 0.4, 0.5]
    if knob == "open_delta_weight":
        return [0.85, 0.7, 0.5]
    raise KeyError(knob)


class Trial:
    """One workload on the device: particles, FP64 reference accelerations on
    sampled particles, and timing of parameter settings."""

    def __init__(self, workload: str, form: int, samples: int = 1024, seed: int = 5):
        self.w = WORKLOADS[workload]
        self.form = form
        self.pm, self.vr, self.sizes = self.w.make()
        self.n = len(self.pm)
        self.nsys = len(self.sizes) if self.sizes else 1
        rng = np.random.default_rng(seed)
        self.samples = np.sort(rng.choice(self.n, size=min(samples, self.n), replace=False)).astype(
            np.uint32)
        self.direct = None

    def params(self, knobs: dict) -> L.Params:
        return default_params(L.PRESET_PHYSICAL, form=self.form, **self.w.physics, **knobs)

    def run(self, knobs: dict, steps: int, warmup: int = 3) -> dict:
        import torch

        sim = Simulation(self.params(knobs), max_n=self.n, max_systems=self.nsys)
        try:
            if self.sizes:
                sim.upload_systems(self.pm, self.vr, self.sizes)
            else:
                sim.upload(self.pm, self.vr)
            sim.draw(0.0, warmup)
            sim.synchronize()
            if self.direct is None:
                self.direct = sim.direct_accel_f64(self.samples)
            stream = torch.cuda.ExternalStream(sim.stream)
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            with torch.cuda.stream(stream):
                ev[0].record(stream)
                sim.draw(0.0, steps)
                ev[1].record(stream)
            sim.synchronize()
            step_ms = ev[0].elapsed_time(ev[1]) / steps
            # The sort stage alone (median of three eager stage sequences).
            sort_ms = []
            for _ in range(3):
                e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
                with torch.cuda.stream(stream):
                    sim.generate_morton_codes()
                    e[0].record(stream)
                    sim.sort()
                    e[1].record(stream)
                    sim.build_tree()
                    sim.barnes_hut()
                    sim.update_spheres(0.0)
                sim.synchronize()
                sort_ms.append(e[0].elapsed_time(e[1]))
            sim.generate_morton_codes()
            sim.sort()
            sim.build_tree()
            sim.barnes_hut()
            acc = sim.read_accel()
            sim.update_spheres(0.0)
            err = np.linalg.norm(acc[self.samples, :3] - self.direct, axis=1) / np.linalg.norm(
                self.direct, axis=1)
        finally:
            sim.close()
        return {"knobs": dict(knobs), "ms": step_ms, "sort_ms": float(np.median(sort_ms)),
                "median_error": float(np.median(err))}


def tune(workload: str, form: str, target: float = 1e-3, steps: int | None = None,
         log=print) -> dict:
    t = Trial(workload, FORMS[form])
    start = {"lbits": t.w.lbits, "bucket": 16, "group_size": 32, "block_warps": 4,
             "sort_variant": 0, "far_ratio": 0.0, "open_delta_weight": 1.0}
    if not steps:
        # About 60 ms of timed steps per trial.
        steps = int(np.clip(60.0 / t.run(start, 3)["ms"], 3, 60))
    best = t.run(start, steps)
    trials = [best]
    bound = max(target, 1.02 * best["median_error"])
    # Accuracy knobs: within 0.8 x the target, or no more than 2% above the
    # starting error where that error is already set by theta (above 0.8 x).
    acc_bound = max(0.8 * target, 1.02 * best["median_error"])
    log(f"{workload}/{form} start {start}: {best['ms']:.3f} ms, error {best['median_error']:.3g}")
    nmax = max(t.sizes) if t.sizes else t.n

    def sweep(knob, limit):
        nonlocal best
        for v in candidates(knob, nmax):
            if knob == "lbits" and 3 * v + (t.nsys - 1).bit_length() > 64:
                continue
            if v == best["knobs"][knob]:
                continue
            r = t.run(dict(best["knobs"], **{knob: v}), steps)
            trials.append(r)
            key = "sort_ms" if knob == "sort_variant" else "ms"
            better = r[key] < best[key] and r["median_error"] <= limit
            log(f"  {knob}={v}: {r['ms']:.3f} ms (sort {r['sort_ms']:.3f}), error "
                f"{r['median_error']:.3g}{'  <- best' if better else ''}")
            if better:
                best = r

    perf = [k for k in KNOBS if k not in ACCURACY_KNOBS]
    for knob in perf:
        sweep(knob, bound)
    # The accuracy knobs share one error budget: every (open_delta_weight,
    # far_ratio) pair, far_ratio rising until the error leaves the bound.
    base = dict(best["knobs"])
    for w in [1.0] + candidates("open_delta_weight", nmax):
        for f in [0.0] + candidates("far_ratio", nmax):
            k = dict(base, open_delta_weight=w, far_ratio=f)
            if k == best["knobs"]:
                continue
            r = t.run(k, steps)
            trials.append(r)
            ok = r["median_error"] <= acc_bound
            better = ok and r["ms"] < best["ms"]
            log(f"  open_delta_weight={w}, far_ratio={f}: {r['ms']:.3f} ms, error "
                f"{r['median_error']:.3g}{'  <- best' if better else ''}")
            if better:
                best = r
            if not ok:
                break
    # The tree and launch knobs again, around the chosen accuracy knobs
    # (group boxes now also decide which nodes are far: the accuracy bound).
    for knob in ("lbits", "bucket", "group_size", "block_warps"):
        sweep(knob, acc_bound)
    return {"workload": workload, "form": form, "n": t.n, "knobs": best["knobs"],
            "ms": best["ms"], "sort_ms": best["sort_ms"], "median_error": best["median_error"],
            "error_bound": bound, "accuracy_knob_bound": acc_bound, "steps_timed": steps,
            "trials": trials}


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
    ap.add_argument("--out", type=Path, default=TUNED_PATH)
    args = ap.parse_args(argv)
    prev = json.loads(args.out.read_text()) if args.out.exists() else {"results": {}}
    results = prev.get("results", {})
    for wl in args.workloads.split(","):
        for form in args.forms.split(","):
            r = tune(wl, form, args.target)
            results[f"{wl}/{form}"] = r
            out = {"device": torch.cuda.get_device_name(),
                   "sms": torch.cuda.get_device_properties(0).multi_processor_count,
                   "when": datetime.datetime.now(datetime.timezone.utc).isoformat(timespec="seconds"),
                   "method": "coordinate descent over " + ", ".join(KNOBS) +
                             "; step time by CUDA events over graph-replayed steps (dt = 0)",
                   "results": results}
            args.out.write_text(json.dumps(out, indent=1) + "\n")
    return 0


if __name__ == "__main__":
    sys.exit(main())
