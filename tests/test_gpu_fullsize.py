"""Parity at the benchmark configurations' full sizes.

One step of each benchmark workload at its real N, through the C ABI, with
the knobs the benchmark uses (astro_gb300/tuned.json, the entry searched at
the quoted tree depth where there is one), in the IEEE-exact form: keys,
permutation, layer sizes/offsets/live counts, node records and
accelerations must equal the CPU restatement's bit for bit, and so must the
interaction, visit and far-node counts. Where the benchmark runs the fast
form, the same step in that form must stay within the parity tolerance
(per particle |a_gpu - a_cpu| <= 2e-5 |a_cpu| + 1e-6 median|a_cpu|) with
identical counts.

C5 at lbits 21 has 2.35e8 node slots: its nodes are compared on windows
(the first 4,194,304 slots, and 262,144 slots at the start of every layer)
rather than held whole as 128-byte records.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ACC_RTOL = 2e-5
ACC_ATOL_REL = 1e-6


def _params(ag, L, workload, form, lbits):
    from astro_gb300 import autotune
    from astro_gb300.workloads import WORKLOADS

    w = WORKLOADS[workload]
    res = autotune.load()
    entry = res.get(autotune.result_key(workload, form, lbits)) or \
        res.get(autotune.result_key(workload, form)) or {}
    k = dict(entry.get("knobs", {}))
    if lbits is not None:
        k["lbits"] = lbits
    k.setdefault("lbits", w.lbits)
    f = L.FORM_PRECISION if form == "precision" else L.FORM_PLAIN
    return w, ag.default_params(L.PRESET_PHYSICAL, form=f, **k, **w.physics)


def _gpu_step(ag, p, pm, vr, sizes, dt, windows):
    with ag.Simulation(p, max_n=len(pm), max_systems=len(sizes) if sizes else 1) as sim:
        if sizes:
            sim.upload_systems(pm, vr, sizes)
        else:
            sim.upload(pm, vr)
        sim.draw(dt, 1)
        codes, sorted_codes, idx = sim.read_keys()
        lsizes, offsets, counts = sim.tree_info()
        out = dict(codes=codes, sorted_codes=sorted_codes, sorted_indices=idx,
                   layer_sizes=lsizes, layer_offsets=offsets, layer_counts=counts,
                   acc4=sim.read_accel())
        out["nodes"] = ([sim.read_nodes()] if windows is None
                        else [sim.read_nodes(a, c) for a, c in windows])
        out["interactions"], out["node_visits"] = sim.read_stats()
        out["far_nodes"], out["far_interactions"] = sim.read_far_stats()
        out["pm"], out["vr"] = sim.download()
    return out


def _windows(lbits, n):
    """Node windows (first slot, count) for trees too large to compare whole
    (None: every slot): the first 4,194,304 slots and 262,144 slots at the
    start of every layer."""
    if lbits < 21:
        return None
    sizes = [min(n, 1 << min(40, 3 * (lbits - l))) for l in range(lbits + 1)]
    offsets = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    return [(0, 1 << 22)] + [(int(o), min(262144, int(s))) for o, s in zip(offsets[1:], sizes[1:])]


def _compare(gpu, ref_nodes, ref, exact):
    for k in ["codes", "sorted_codes", "sorted_indices", "layer_sizes", "layer_offsets",
              "layer_counts"]:
        assert np.array_equal(gpu[k], ref[k]), k
    for g_nodes, r_nodes in zip(gpu["nodes"], ref_nodes):
        assert g_nodes.shape == r_nodes.shape
        for f in ["mortonCode", "children", "layer", "totalMass", "centerOfMass"]:
            assert np.array_equal(g_nodes[f], r_nodes[f]), f
        assert np.array_equal(g_nodes, r_nodes)
    for key in ("interactions", "node_visits", "far_nodes", "far_interactions"):
        assert gpu[key] == ref[key], key
    if exact:
        assert np.array_equal(gpu["acc4"], ref["acc4"])
    else:
        a = ref["acc4"][:, :3].astype(np.float64)
        d = np.linalg.norm(gpu["acc4"][:, :3].astype(np.float64) - a, axis=1)
        na = np.linalg.norm(a, axis=1)
        ok = d <= ACC_RTOL * na + ACC_ATOL_REL * np.median(na)
        assert ok.all(), f"{(~ok).sum()} particles outside tolerance, worst " \
                         f"{(d / np.maximum(na, 1e-30)).max():.3e}"


@pytest.mark.parametrize("workload,form,lbits,fast", [
    ("c2", "plain", None, True),       # 524,288: disk + bulge, the tuned knobs
    ("c3", "precision", None, False),  # 4,194,304: two Plummer spheres, precision form
    ("c4", "precision", None, False),  # 256 systems (8-bit system field), precision form
    ("c5", "plain", 6, True),          # 16,777,216: the reference's 7 layers
    ("c5", "plain", 21, False),        # 16,777,216: 63-bit keys, 8 sort passes
])
def test_benchmark_configuration_at_full_size(native, oracle, workload, form, lbits, fast):
    ag = native
    L = ag.layouts
    w, p = _params(ag, L, workload, form, lbits)
    pm, vr, sizes = w.make()
    n = len(pm)
    windows = _windows(p.lbits, n) if not sizes else None
    p_exact = p.replace(flags=p.flags | L.FLAG_IEEE_EXACT)
    gpu = _gpu_step(ag, p_exact, pm.copy(), vr.copy(), sizes, w.dt, windows)
    pm_o, vr_o = pm.copy(), vr.copy()
    if windows is None:
        ref = oracle.phys_run(p_exact, pm_o, vr_o, sizes=sizes, dt=w.dt, steps=1)
        ref_nodes = [ref["nodes"]]
    else:
        slots = np.concatenate([np.arange(a, a + c, dtype=np.uint64) for a, c in windows])
        ref = oracle.phys_run(p_exact, pm_o, vr_o, sizes=sizes, dt=w.dt, steps=1, nodes=slots)
        ref_nodes = np.split(ref["nodes"], np.cumsum([c for _, c in windows])[:-1])
    _compare(gpu, ref_nodes, ref, exact=True)
    assert np.array_equal(gpu["pm"], pm_o) and np.array_equal(gpu["vr"], vr_o)
    if fast:
        fast_out = _gpu_step(ag, p, pm.copy(), vr.copy(), sizes, w.dt, windows)
        _compare(fast_out, ref_nodes, ref, exact=False)
