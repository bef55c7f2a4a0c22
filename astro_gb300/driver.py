"""Headless step loop: the reference's frame loop without the render pass.

Renderer (Astro/Renderer.swift) builds a scene in makeSpheres (:441-493),
rebuilds it on resetSimulation (:148-152) and advances it once per frame in
draw (:495-553). This driver does the same from the command line: it
generates a seeded scene (or resumes from a state file), runs the step on the
GPU, and writes state files at a fixed step interval, so a run can be stopped
and continued bit-exactly.

  python -m astro_gb300.driver --scene disk_bulge --n 524288 --steps 1000 \\
      --dt 5e-4 --save-every 250 --out runs/disk
  python -m astro_gb300.driver --resume runs/disk/step_000500.state --steps 500 \\
      --out runs/disk

Scenes: reference (the reference's stars/planets/dust scene, REFERENCE
preset), plummer, disk_bulge, two_plummer, uniform_cube (PHYSICAL preset).
Each save prints one JSON line with the step, the simulated time, the state
file and the mean step time since the previous save.
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

from . import ic
from . import layouts as L
from .simulation import Simulation, default_params

SCENES = ("reference", "plummer", "disk_bulge", "two_plummer", "uniform_cube")


def make_scene(args) -> tuple[Simulation, float]:
    """A new context holding the generated scene, and its default dt."""
    if args.scene == "reference":
        p = default_params(L.PRESET_REFERENCE)
        pm, vr, ct = ic.reference_scene(args.stars, args.planets, args.n - args.stars - args.planets,
                                        seed=args.seed)
        sim = Simulation(p, max_n=args.n)
        sim.upload(pm, vr, ct, n_tree=args.stars + args.planets)
        return sim, 1.0 / 60.0
    form = L.FORM_PRECISION if args.form == "precision" else L.FORM_PLAIN
    p = default_params(L.PRESET_PHYSICAL, form=form, softening=args.eps, theta=args.theta,
                       lbits=args.lbits)
    pm, vr = getattr(ic, args.scene)(args.n, args.seed)
    sim = Simulation(p, max_n=args.n)
    sim.upload(pm, vr)
    return sim, 1e-3


def run(args, log=print) -> list[dict]:
    out = Path(args.out)
    out.mkdir(parents=True, exist_ok=True)
    if args.resume:
        sim, step, t = Simulation.load_state(args.resume)
        dt = args.dt
        if dt is None:
            raise SystemExit("--dt is required with --resume")
    else:
        sim, dt_default = make_scene(args)
        step, t = 0, 0.0
        dt = args.dt if args.dt is not None else dt_default
    records = []
    with sim:
        end = step + args.steps
        every = args.save_every or args.steps
        while step < end:
            k = min(every - step % every, end - step)
            t0 = time.perf_counter()
            sim.draw(dt, k)
            sim.synchronize()
            wall = time.perf_counter() - t0
            step += k
            t += k * dt
            if step % every == 0 or step == end:
                path = out / f"step_{step:06d}.state"
                sim.save_state(path, step, t)
                rec = {"step": step, "time": t, "state": str(path),
                       "ms_per_step": 1e3 * wall / k, "n": sim.n}
                records.append(rec)
                log(json.dumps(rec))
    return records


def parse(argv=None):
    ap = argparse.ArgumentParser(description="Headless Barnes-Hut step loop with state files.")
    ap.add_argument("--scene", choices=SCENES, default="disk_bulge")
    ap.add_argument("--n", type=int, default=65536)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--stars", type=int, default=5)
    ap.add_argument("--planets", type=int, default=200)
    ap.add_argument("--form", choices=["plain", "precision"], default="plain")
    ap.add_argument("--eps", type=float, default=0.005)
    ap.add_argument("--theta", type=float, default=0.7)
    ap.add_argument("--lbits", type=int, default=14)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--dt", type=float, default=None)
    ap.add_argument("--save-every", type=int, default=0)
    ap.add_argument("--out", default="runs")
    ap.add_argument("--resume", default=None, help="state file to continue from")
    return ap.parse_args(argv)


def main(argv=None) -> int:
    run(parse(argv))
    return 0


if __name__ == "__main__":
    sys.exit(main())
