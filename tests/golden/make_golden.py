"""Generate the hand-derived golden vectors of the Barnes-Hut step.

The reference (osbo/astro) ships no golden vectors, fixtures or kernel tests,
and it cannot run here (Swift + Metal on macOS). These fixtures are derived
from the reference source by hand and by plain Python arithmetic that restates
each formula independently of both the CPU restatement (oracle/) and the CUDA
path, so both are checked against them:

  morton.json     generateMortonCodes (MortonCode.metal:26-52): (u32)(p+1e6),
                  masked to 21 bits, bit i of x/y/z -> key bit 3i/3i+1/3i+2,
                  >> 45; including the 0x1FFFFF wrap and the saturation at 0.
  octants.json    eight bodies, one per octant at the top level: keys, live
                  node counts per layer (Renderer.swift:373-386 capacity),
                  root children and root centre of mass.
  two_body.json   barnesHut (BarnesHut.metal:22-101) for two bodies: the
                  monopole g m d / (r^2 + 0.01)^1.5, the clamp at 1e5, the
                  r^2 > 50 cut and the self-leaf skip.
  last_leaf.json  aggregateLeafNodes' last run ending at numUnique
                  (Octree.metal:71) with duplicate keys.
  sort.json       a stable sort of keys with duplicates.

Run: python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
F32 = np.float32


def sat_u32(f: np.float32) -> int:
    f = float(f)
    if not f > 0.0:
        return 0
    if f >= 4294967296.0:
        return 0xFFFFFFFF
    return int(f)


def ref_key(x: float, y: float, z: float, lbits: int = 6, offset: float = 1e6) -> int:
    q = [sat_u32(F32(F32(c) + F32(offset))) & 0x1FFFFF for c in (x, y, z)]
    key = 0
    for i in range(21):
        for axis in range(3):
            if (q[axis] >> i) & 1:
                key |= 1 << (3 * i + axis)
    return key >> (63 - 3 * lbits)


def morton() -> dict:
    cases = []
    pts = [(0.0, 0.0, 0.0), (-1e6, -1e6, -1e6), (-2e6, 5.0, 1.0), (1.1e6, 0.0, 0.0),
           (4.3e9, 0.0, 0.0), (1097151.0, 1097151.0, 1097151.0), (32767.0 - 1e6, 0.0, 0.0),
           (32768.0 - 1e6, 0.0, 0.0), (123456.0, -654321.0, 999999.0)]
    for p in pts:
        cases.append({"pos": list(p), "key": ref_key(*p)})
    # Hand check: 1e6 >> 15 = 30 = 0b011110, so the origin maps to bits 1..4
    # set on all three axes: 7<<3 | 7<<6 | 7<<9 | 7<<12 = 32760.
    assert cases[0]["key"] == 32760
    # -1e6 + 1e6 = 0 on every axis -> key 0; -2e6 + 1e6 < 0 saturates to 0.
    assert cases[1]["key"] == 0
    # 2.1e6 wraps: (2100000 & 0x1FFFFF) >> 15 = 2848 >> 15 = 0.
    assert (ref_key(1.1e6, 0, 0) >> 0) & 0b1 == 0
    # 4.3e9 saturates to 0xFFFFFFFF -> 0x1FFFFF -> top six bits all set on x.
    assert cases[4]["key"] & 0b001001001001001001 == 0b001001001001001001
    return {"lbits": 6, "offset": 1e6, "cases": cases}


def octants() -> dict:
    # q = 16 (0b010000) and q = 48 (0b110000) differ only in the top bit, so
    # the eight bodies split at the root and nowhere else.
    lo = 16 * 32768 + 100 - 1e6
    hi = 48 * 32768 + 100 - 1e6
    pos, keys = [], []
    for octant in [5, 0, 3, 6, 1, 7, 2, 4]:
        hx, hy, hz = octant & 1, (octant >> 1) & 1, (octant >> 2) & 1
        p = (hi if hx else lo, hi if hy else lo, hi if hz else lo)
        pos.append(p)
        keys.append(ref_key(*p))
        assert keys[-1] == 0x7000 | (octant << 15)
    order = sorted(range(8), key=lambda i: keys[i])
    counts = [8, 8, 8, 8, 8, 8, 1]
    sizes = [8, 8, 8, 8, 8, 8, 1]
    offsets = [0, 8, 16, 24, 32, 40, 48]
    root = 48
    root_children = [40 + k for k in range(8)]
    com = [sum(p[a] for p in pos) / 8.0 for a in range(3)]
    return {"positions": pos, "mass": 1.0, "keys": keys, "sorted_indices": order,
            "layer_counts": counts, "layer_sizes": sizes, "layer_offsets": offsets,
            "root": root, "root_children": root_children, "root_mass": 8.0, "root_com": com}


def two_body() -> dict:
    # Leaf cells are 2^15 = 32768 units wide (lbits = 6). Body 0 at x0, body 1
    # at x0 + d on the x axis; force on each body.
    g, soft = 1e11, 0.01
    cases = []
    for x0, d, m, kind in [(0.0, 40000.0, 1.0, "monopole"),     # leaves 30 and 31
                           (0.0, 40000.0, 1e4, "clamped"),      # 6.25e5 -> 1e5
                           (-967232.5, 5.0, 1.0, "cut"),        # leaves 0 and 1, r^2 < 50
                           (0.0, 1000.0, 1.0, "self")]:         # one leaf: both skip it
        assert (ref_key(x0, 0, 0) == ref_key(x0 + d, 0, 0)) == (kind == "self")
        if kind in ("cut", "self"):
            fx = 0.0
        else:
            r2 = d * d + soft
            fx = min(max(g * m * d / (r2 * np.sqrt(r2)), -1e5), 1e5)
        cases.append({"x0": x0, "d": d, "m": m, "kind": kind, "fx0": fx, "fx1": -fx})
    return {"g": g, "softening": soft, "cases": cases}


def last_leaf() -> dict:
    # Bodies 0 and 1 share a position (one key), body 2 sits in another leaf
    # with a larger key. numUnique = 2; the last leaf starts at sorted slot 2
    # and the reference ends it at numUnique = 2: an empty range.
    pos = [(0.0, 0.0, 0.0), (0.0, 0.0, 0.0), (500000.0, 500000.0, 500000.0)]
    masses = [1.0, 2.0, 4.0]
    return {"positions": pos, "masses": masses, "reference_leaf_mass": [3.0, 0.0],
            "reference_leaf_com": [[0.0, 0.0, 0.0], [0.0, 0.0, 0.0]],
            "fixed_leaf_mass": [3.0, 4.0]}


def sort() -> dict:
    keys = [3, 1, 3, 1, 0, 2, 3, 0]
    perm = sorted(range(len(keys)), key=lambda i: (keys[i], i))
    assert perm == [4, 7, 1, 3, 5, 0, 2, 6]
    return {"keys": keys, "perm": perm}


def main() -> None:
    for name, fn in [("morton", morton), ("octants", octants), ("two_body", two_body),
                     ("last_leaf", last_leaf), ("sort", sort)]:
        (HERE / f"{name}.json").write_text(json.dumps(fn(), indent=1) + "\n")
        print("wrote", name)


if __name__ == "__main__":
    main()
