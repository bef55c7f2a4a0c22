"""Parity of the CUDA path (through the C ABI) with the CPU restatement.

Bit-exact: Morton keys, sort permutation, layer sizes/offsets/live counts,
node records (codes, children, layers, masses, centres of mass) and, in the
REFERENCE preset and the IEEE-exact PHYSICAL traversal, accelerations and the
integrated state.
Tolerance: the fast PHYSICAL traversal (rsqrt and FMA) differs from the
restatement only by rounding in each interaction; its accelerations must
satisfy |a_gpu - a_cpu| <= 2e-5 |a_cpu| + 1e-6 median|a_cpu| per particle,
and the opening decisions (interaction and visit counts) must be identical.
"""
import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
ACC_RTOL = 2e-5
ACC_ATOL_REL = 1e-6


def load(name):
    return json.loads((GOLDEN / f"{name}.json").read_text())


@pytest.fixture(scope="module")
def ag(native):
    return native


def particles(L, pos, masses=None):
    pm, vr = L.empty_particles(len(pos))
    pm["position"] = np.asarray(pos, np.float32)
    pm["mass"] = 1.0 if masses is None else np.asarray(masses, np.float32)
    return pm, vr


def run_gpu(ag, params, pm, vr, ct=None, n_tree=None, dt=0.0, steps=1, sizes=None):
    with ag.Simulation(params, max_n=len(pm), max_systems=max(1, len(sizes or [1]))) as sim:
        if sizes is not None:
            sim.upload_systems(pm, vr, sizes)
        else:
            sim.upload(pm, vr, ct, n_tree=n_tree)
        sim.draw(dt, steps)
        codes, sorted_codes, idx = sim.read_keys()
        sizes_, offsets, counts = sim.tree_info()
        out = dict(codes=codes, sorted_codes=sorted_codes, sorted_indices=idx,
                   layer_sizes=sizes_, layer_offsets=offsets, layer_counts=counts,
                   nodes=sim.read_nodes(), acc4=sim.read_accel())
        out["interactions"], out["node_visits"] = sim.read_stats()
        out["far_nodes"], out["far_interactions"] = sim.read_far_stats()
        out["pm"], out["vr"] = sim.download()
    return out


def assert_tree_equal(gpu, ref):
    for k in ["codes", "sorted_codes", "sorted_indices", "layer_sizes", "layer_offsets",
              "layer_counts"]:
        assert np.array_equal(gpu[k], ref[k]), k
    assert gpu["nodes"].shape == ref["nodes"].shape
    for f in ["mortonCode", "children", "layer", "totalMass", "centerOfMass"]:
        assert np.array_equal(gpu["nodes"][f], ref["nodes"][f]), f
    assert np.array_equal(gpu["nodes"], ref["nodes"])


def acc_close(gpu, ref):
    a = ref[:, :3].astype(np.float64)
    d = np.linalg.norm(gpu[:, :3].astype(np.float64) - a, axis=1)
    na = np.linalg.norm(a, axis=1)
    tol = ACC_RTOL * na + ACC_ATOL_REL * np.median(na)
    return d <= tol, d / np.maximum(na, 1e-30)


# ------------------------------------------------------------ REFERENCE --

def test_reference_golden_morton_and_octants(ag, oracle):
    L = ag.layouts
    p = ag.default_params(L.PRESET_REFERENCE)
    g = load("morton")
    pm, vr = particles(L, [c["pos"] for c in g["cases"]])
    out = run_gpu(ag, p, pm, vr)
    assert [int(c) for c in out["codes"]] == [c["key"] for c in g["cases"]]
    g = load("octants")
    pm, vr = particles(L, g["positions"])
    out = run_gpu(ag, p, pm, vr)
    assert [int(k) for k in out["codes"]] == g["keys"]
    assert [int(i) for i in out["sorted_indices"]] == g["sorted_indices"]
    assert list(out["layer_counts"]) == g["layer_counts"]
    root = out["nodes"][g["root"]]
    assert list(root["children"]) == g["root_children"] and root["totalMass"] == 8.0
    ref = oracle.ref_run(p, pm.copy(), vr.copy(), dt=0.0, steps=1)
    assert_tree_equal(out, ref)


@pytest.mark.parametrize("case", range(4))
def test_reference_golden_two_body(ag, oracle, case):
    L = ag.layouts
    c = load("two_body")["cases"][case]
    pm, vr = particles(L, [(c["x0"], 0, 0), (c["x0"] + c["d"], 0, 0)], [c["m"], c["m"]])
    out = run_gpu(ag, ag.default_params(L.PRESET_REFERENCE), pm, vr)
    assert out["acc4"][0, 0] == pytest.approx(c["fx0"], rel=1e-5)
    assert out["acc4"][1, 0] == pytest.approx(c["fx1"], rel=1e-5)


def test_reference_golden_last_leaf(ag):
    L = ag.layouts
    g = load("last_leaf")
    pm, vr = particles(L, g["positions"], g["masses"])
    out = run_gpu(ag, ag.default_params(L.PRESET_REFERENCE), pm, vr)
    assert list(out["nodes"][:2]["totalMass"]) == g["reference_leaf_mass"]
    out = run_gpu(ag, ag.default_params(L.PRESET_PHYSICAL), pm, vr)
    assert list(out["nodes"][:2]["totalMass"]) == g["fixed_leaf_mass"]


def test_reference_scene_bit_exact(ag, oracle):
    from astro_gb300 import ic

    L = ag.layouts
    p = ag.default_params(L.PRESET_REFERENCE)
    pm, vr, ct = ic.reference_scene(5, 200, 5000, seed=21)
    out = run_gpu(ag, p, pm, vr, ct, n_tree=205, dt=1.0 / 60, steps=3)
    pm_o, vr_o = pm.copy(), vr.copy()
    ref = oracle.ref_run(p, pm_o, vr_o, ct, n_tree=205, dt=1.0 / 60, steps=3, split_passes=64)
    assert_tree_equal(out, ref)
    # The stars light the tree: emitted colours and centres are part of the
    # compared records (Octree.metal:75-106,147-187).
    assert (out["nodes"]["emittedColor"][:, 3] > 0).sum() >= 5
    assert np.array_equal(out["nodes"]["emittedColorCenter"], ref["nodes"]["emittedColorCenter"])
    assert np.array_equal(out["acc4"], ref["acc4"])
    assert np.array_equal(out["pm"], pm_o) and np.array_equal(out["vr"], vr_o)


def test_reference_plummer_all_in_tree(ag, oracle):
    from astro_gb300 import ic

    L = ag.layouts
    p = ag.default_params(L.PRESET_REFERENCE)
    pm, vr = ic.plummer(16384, seed=1001)
    pm["position"] *= 4e4  # into the reference's units (positions ~1e6)
    out = run_gpu(ag, p, pm, vr, dt=1e-3, steps=2)
    pm_o, vr_o = pm.copy(), vr.copy()
    ref = oracle.ref_run(p, pm_o, vr_o, dt=1e-3, steps=2, split_passes=18)
    assert_tree_equal(out, ref)
    assert np.array_equal(out["acc4"], ref["acc4"])
    assert np.array_equal(out["pm"], pm_o)


# ------------------------------------------------------------- PHYSICAL --

WALKS = {
    "group": lambda L: L.FLAG_OPEN_DELTA | L.FLAG_QUADRUPOLE,
    "group-monopole": lambda L: 0,
    "particle": lambda L: L.FLAG_PER_PARTICLE | L.FLAG_OPEN_DELTA | L.FLAG_QUADRUPOLE,
    "particle-monopole": lambda L: L.FLAG_PER_PARTICLE,
}


@pytest.mark.parametrize("walk,lbits", [("group", 6), ("group", 10), ("group", 21),
                                        ("group-monopole", 21), ("particle", 21),
                                        ("particle-monopole", 6)])
def test_physical_exact_bit_exact(ag, oracle, walk, lbits):
    from astro_gb300 import ic

    L = ag.layouts
    p = ag.default_params(L.PRESET_PHYSICAL, lbits=lbits, flags=WALKS[walk](L) | L.FLAG_IEEE_EXACT)
    pm, vr = ic.plummer(16384, seed=1001)
    out = run_gpu(ag, p, pm, vr, dt=1e-3, steps=3)
    pm_o, vr_o = pm.copy(), vr.copy()
    ref = oracle.phys_run(p, pm_o, vr_o, dt=1e-3, steps=3)
    assert_tree_equal(out, ref)
    assert np.array_equal(out["acc4"], ref["acc4"])
    assert out["interactions"] == ref["interactions"] and out["node_visits"] == ref["node_visits"]
    assert np.array_equal(out["pm"], pm_o) and np.array_equal(out["vr"], vr_o)


@pytest.mark.parametrize("walk,warps,persistent", [("group", 4, False), ("group", 8, False),
                                                   ("group-monopole", 4, False),
                                                   ("particle", 4, False), ("particle", 2, True),
                                                   ("particle-monopole", 8, False)])
def test_physical_fast_within_tolerance(ag, oracle, walk, warps, persistent):
    from astro_gb300 import ic

    L = ag.layouts
    flags = WALKS[walk](L) | (L.FLAG_PERSISTENT if persistent else 0)
    p = ag.default_params(L.PRESET_PHYSICAL, flags=flags, block_warps=warps, softening=0.005,
                          lbits=21)
    pm, vr = ic.disk_bulge(32768, seed=1002)
    out = run_gpu(ag, p, pm, vr, dt=5e-4, steps=1)
    ref = oracle.phys_run(p, pm.copy(), vr.copy(), dt=5e-4, steps=1)
    assert_tree_equal(out, ref)
    ok, rel = acc_close(out["acc4"], ref["acc4"])
    assert ok.all(), f"{(~ok).sum()} particles outside tolerance, worst {rel.max():.3e}"
    assert out["interactions"] == ref["interactions"] and out["node_visits"] == ref["node_visits"]


@pytest.mark.parametrize("group_size,sort_variant,form", [(8, 1, 0), (16, 4, 1), (1, 7, 0),
                                                         (32, 6, 1), (5, 2, 0), (24, 3, 0),
                                                         (12, 5, 0), (32, 8, 0), (20, 9, 1),
                                                         (16, 10, 0), (48, 11, 1), (64, 12, 0)])
def test_group_size_and_sort_variant_bit_exact(ag, oracle, group_size, sort_variant, form):
    """Particles per warp and the sort's pass kernel are tuning knobs: every
    setting must give the oracle's tree and accelerations bit for bit."""
    from astro_gb300 import ic

    L = ag.layouts
    p = ag.default_params(L.PRESET_PHYSICAL, lbits=10, form=form, group_size=group_size,
                          sort_variant=sort_variant, flags=WALKS["group"](L) | L.FLAG_IEEE_EXACT)
    pm, vr = ic.plummer(16384, seed=1001)
    out = run_gpu(ag, p, pm, vr, dt=1e-3, steps=2)
    pm_o, vr_o = pm.copy(), vr.copy()
    ref = oracle.phys_run(p, pm_o, vr_o, dt=1e-3, steps=2)
    assert_tree_equal(out, ref)
    assert np.array_equal(out["acc4"], ref["acc4"])
    assert out["interactions"] == ref["interactions"] and out["node_visits"] == ref["node_visits"]
    assert np.array_equal(out["pm"], pm_o) and np.array_equal(out["vr"], vr_o)


@pytest.mark.parametrize("group_size,form", [(4, 0), (12, 0), (16, 1), (7, 1)])
def test_physical_fast_small_groups_within_tolerance(ag, oracle, group_size, form):
    """Groups of at most 16 run as several copies that split the source
    lists; the sum must stay within the fast path's tolerance."""
    from astro_gb300 import ic

    L = ag.layouts
    p = ag.default_params(L.PRESET_PHYSICAL, softening=0.005, lbits=14, group_size=group_size,
                          form=form)
    pm, vr = ic.disk_bulge(32768, seed=1002)
    out = run_gpu(ag, p, pm, vr, dt=5e-4, steps=1)
    ref = oracle.phys_run(p, pm.copy(), vr.copy(), dt=5e-4, steps=1)
    assert_tree_equal(out, ref)
    ok, rel = acc_close(out["acc4"], ref["acc4"])
    assert ok.all(), f"{(~ok).sum()} particles outside tolerance, worst {rel.max():.3e}"
    assert out["interactions"] == ref["interactions"] and out["node_visits"] == ref["node_visits"]


def test_physical_precision_form_bit_exact(ag, oracle):
    from astro_gb300 import ic

    L = ag.layouts
    p = ag.default_params(L.PRESET_PHYSICAL, form=L.FORM_PRECISION,
                          flags=WALKS["group"](L) | L.FLAG_IEEE_EXACT, softening=0.002, lbits=10)
    pm, vr = ic.two_plummer(16384, seed=1003)
    out = run_gpu(ag, p, pm, vr, dt=1e-3, steps=3)
    pm_o, vr_o = pm.copy(), vr.copy()
    ref = oracle.phys_run(p, pm_o, vr_o, dt=1e-3, steps=3)
    assert_tree_equal(out, ref)
    assert np.array_equal(out["acc4"], ref["acc4"])
    assert np.array_equal(out["pm"], pm_o) and np.array_equal(out["vr"], vr_o)


@pytest.mark.parametrize("walk,persistent", [("group", False), ("particle", False),
                                             ("particle-monopole", True)])
def test_physical_batched_bit_exact(ag, oracle, walk, persistent):
    from astro_gb300 import ic

    L = ag.layouts
    sizes = [1, 2, 31, 33, 1024, 5000, 64, 3, 4096, 777]
    parts = [ic.plummer(s, seed=1004, a=0.5 + 0.1 * k, system=k) for k, s in enumerate(sizes)]
    pm = np.concatenate([a for a, _ in parts])
    vr = np.concatenate([b for _, b in parts])
    flags = WALKS[walk](L) | L.FLAG_IEEE_EXACT | (L.FLAG_PERSISTENT if persistent else 0)
    p = ag.default_params(L.PRESET_PHYSICAL, flags=flags)
    out = run_gpu(ag, p, pm, vr, dt=1e-3, steps=2, sizes=sizes)
    pm_o, vr_o = pm.copy(), vr.copy()
    ref = oracle.phys_run(p, pm_o, vr_o, sizes=sizes, dt=1e-3, steps=2)
    assert_tree_equal(out, ref)
    assert np.array_equal(out["acc4"], ref["acc4"])
    assert np.array_equal(out["pm"], pm_o)


def test_graph_replay_equals_eager(ag):
    from astro_gb300 import ic

    L = ag.layouts
    pm, vr = ic.plummer(20000, seed=5)
    res = []
    for flags in [0, L.FLAG_NO_GRAPH]:
        p = ag.default_params(L.PRESET_PHYSICAL, flags=flags)
        with ag.Simulation(p, max_n=len(pm)) as sim:
            sim.upload(pm, vr)
            sim.draw(1e-3, 5)
            res.append(sim.download())
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1])


def test_stage_calls_equal_step(ag):
    from astro_gb300 import ic

    L = ag.layouts
    pm, vr = ic.plummer(10000, seed=6)
    p = ag.default_params(L.PRESET_PHYSICAL)
    with ag.Simulation(p, max_n=len(pm)) as sim:
        sim.upload(pm, vr)
        sim.draw(1e-3, 1)
        a = sim.download()
    with ag.Simulation(p, max_n=len(pm)) as sim:
        sim.upload(pm, vr)
        sim.generate_morton_codes()
        sim.sort()
        sim.build_tree()
        sim.barnes_hut()
        sim.update_spheres(1e-3)
        b = sim.download()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_upload_download_round_trip_and_errors(ag):
    from astro_gb300 import ic

    L = ag.layouts
    pm, vr = ic.uniform_cube(1000, seed=1)
    p = ag.default_params(L.PRESET_PHYSICAL)
    with ag.Simulation(p, max_n=1000) as sim:
        with pytest.raises(ag.AstroError) as e:
            sim.barnes_hut()
        assert e.value.status == -5
        sim.upload(pm, vr)
        got_pm, got_vr = sim.download()
        assert np.array_equal(got_pm["position"], pm["position"])
        assert np.array_equal(got_pm["mass"], pm["mass"])
        assert np.array_equal(got_vr["velocity"], vr["velocity"])
        with pytest.raises(ag.AstroError) as e:
            sim.barnes_hut()
        assert e.value.status == -5
        big_pm, big_vr = ic.uniform_cube(1001, seed=1)
        with pytest.raises(ag.AstroError) as e:
            sim.upload(big_pm, big_vr)
        assert e.value.status == -2


def test_direct_sum_f64_matches_cpu(ag, oracle):
    from astro_gb300 import ic

    L = ag.layouts
    pm, vr = ic.plummer(30000, seed=8)
    p = ag.default_params(L.PRESET_PHYSICAL, softening=0.01)
    samples = np.arange(0, 30000, 97, dtype=np.uint32)
    with ag.Simulation(p, max_n=len(pm)) as sim:
        sim.upload(pm, vr)
        gpu = sim.direct_accel_f64(samples)
    # The context softens with the FP32 value of eps; give the CPU the same.
    cpu = oracle.direct_accel(pm, samples, g=1.0, eps=float(np.float32(0.01)))
    # Both sum 30,000 FP64 terms, in different orders (and the GPU contracts
    # into FMAs); the difference stays near n * 2^-53 times the term sizes.
    assert np.abs(gpu - cpu).max() < 1e-10 * max(1.0, np.abs(cpu).max())


# ----------------------------------------------------------------- sort --

@pytest.mark.parametrize("n", [1, 2, 4095, 4096, 4097, 100003, 1 << 20, 3_000_017])
@pytest.mark.parametrize("key_bits", [18, 26, 63, 64])
def test_radix_sort_matches_stable_argsort(ag, n, key_bits):
    import torch

    from astro_gb300.radix_sort import RadixSort

    rng = np.random.default_rng(n + key_bits)
    hi = (1 << key_bits) if key_bits < 64 else None
    if hi is None:
        keys = rng.integers(0, 1 << 63, n, dtype=np.uint64) * 2 + rng.integers(0, 2, n).astype(np.uint64)
    else:
        keys = rng.integers(0, hi, n, dtype=np.uint64)
    keys[rng.integers(0, n, n // 3 + 1)] = keys[0]  # duplicates
    idx_in = rng.permutation(n).astype(np.uint32)
    dk = torch.from_numpy(keys.view(np.int64)).cuda()
    di = torch.from_numpy(idx_in.view(np.int32)).cuda()
    ok = torch.empty_like(dk)
    oi = torch.empty_like(di)
    s = RadixSort(n, key_bits)
    s.sort(dk, di, ok, oi, n)
    torch.cuda.synchronize()
    want = np.argsort(keys, kind="stable")
    assert np.array_equal(ok.cpu().numpy().view(np.uint64), keys[want])
    assert np.array_equal(oi.cpu().numpy().view(np.uint32), idx_in[want])
    # Inputs untouched.
    assert np.array_equal(dk.cpu().numpy().view(np.uint64), keys)


def test_radix_sort_device_count_and_iota(ag):
    import torch

    from astro_gb300.radix_sort import RadixSort

    rng = np.random.default_rng(1)
    est, count = 50000, 31234
    keys = rng.integers(0, 1 << 18, est, dtype=np.uint64)
    dk = torch.from_numpy(keys.view(np.int64)).cuda()
    ok = torch.full_like(dk, -1)
    oi = torch.full((est,), -1, dtype=torch.int32, device="cuda")
    cnt = torch.tensor([count], dtype=torch.int32, device="cuda")
    s = RadixSort(est, 18)
    s.sort(dk, None, ok, oi, est, cnt)
    torch.cuda.synchronize()
    want = np.argsort(keys[:count], kind="stable")
    assert np.array_equal(ok.cpu().numpy().view(np.uint64)[:count], keys[:count][want])
    assert np.array_equal(oi.cpu().numpy().view(np.uint32)[:count], want.astype(np.uint32))
    # Slots past the count are not written.
    assert (ok.cpu().numpy()[count:] == -1).all()


# ------------------------------------------------ full-size properties --

def test_large_uniform_cube_properties(ag):
    """16.7M bodies at lbits = 21 (63-bit keys): properties that do not need
    the CPU restatement."""
    from astro_gb300 import ic

    L = ag.layouts
    n = 1 << 24
    pm, vr = ic.uniform_cube(n, seed=1005)
    p = ag.default_params(L.PRESET_PHYSICAL, lbits=21, softening=0.001)
    with ag.Simulation(p, max_n=n) as sim:
        sim.upload(pm, vr)
        sim.draw(0.0, 1)
        codes, sorted_codes, idx = sim.read_keys()
        sizes, offsets, counts = sim.tree_info()
        acc = sim.read_accel()
        samples = np.arange(0, n, n // 2048, dtype=np.uint32)
        direct = sim.direct_accel_f64(samples)
        top = sim.read_nodes(int(offsets[-1]), 1)
    assert np.all(sorted_codes[1:] >= sorted_codes[:-1])
    assert np.array_equal(np.sort(idx), np.arange(n, dtype=np.uint32))
    assert np.array_equal(codes[idx], sorted_codes)
    assert counts[-1] == 1 and np.all(counts[1:] <= counts[:-1])
    assert top["totalMass"][0] == pytest.approx(1.0, rel=1e-4)
    err = np.linalg.norm(acc[samples, :3] - direct, axis=1) / np.linalg.norm(direct, axis=1)
    assert np.median(err) < 1e-2


# ------------------------------------------------------------- lighting --

def test_lighting_pass_bit_exact(ag, oracle):
    """lightingPass alone and inside the REFERENCE step (between barnesHut and
    updateSpheres, so it sees the positions before the kick-drift)."""
    from astro_gb300 import ic

    L = ag.layouts
    pm, vr, ct = ic.reference_scene(5, 200, 20000, seed=3)
    n = len(pm)
    p = ag.default_params(L.PRESET_REFERENCE)
    with ag.Simulation(p, max_n=n) as sim:
        sim.upload(pm, vr, ct, n_tree=205)
        sim.lighting_pass(5)
        got = sim.read_colors()
    want = oracle.lighting(pm, ct, 5)
    assert np.array_equal(got["color"], want["color"])
    assert np.array_equal(got["type"], ct["type"])
    lit = want["type"] != 0
    assert (want["color"][lit] != ct["color"][lit]).any()
    # In the step: colours from the positions at the start of the step.
    with ag.Simulation(p, max_n=n) as sim:
        sim.upload(pm, vr, ct, n_tree=205)
        sim.draw(1.0 / 60, 1)
        assert np.array_equal(sim.read_colors()["color"], want["color"])
        moved, _ = sim.download()
    assert not np.array_equal(moved["position"], pm["position"])
    # light_sources = 0 leaves the colours as uploaded.
    with ag.Simulation(p.replace(light_sources=0), max_n=n) as sim:
        sim.upload(pm, vr, ct, n_tree=205)
        sim.draw(1.0 / 60, 1)
        assert np.array_equal(sim.read_colors()["color"], ct["color"])


# ---------------------------------------------------------------- splat --

@pytest.mark.parametrize("width,height,pos", [(320, 240, (0.0, 0.0, 1.8e6)),
                                              (257, 131, (2e5, -1e5, 6e5))])
def test_splat_bit_exact(ag, oracle, width, height, pos):
    """The headless scene pass against its sequential CPU restatement: every
    pixel's colour and depth, after the lighting pass, for the reference's
    camera and a close one (large discs, partly off-screen)."""
    from astro_gb300 import ic
    from astro_gb300.render import reference_camera

    L = ag.layouts
    pm, vr, ct = ic.reference_scene(5, 200, 30000, seed=11)
    n = len(pm)
    cam = reference_camera(width, height, position=pos)
    with ag.Simulation(ag.default_params(L.PRESET_REFERENCE), max_n=n) as sim:
        sim.upload(pm, vr, ct, n_tree=205)
        sim.lighting_pass(5)
        lit = sim.read_colors()
        rgba, depth = sim.splat(cam, width, height)
        # A second call reuses the fragment buffers.
        rgba2, depth2 = sim.splat(cam, width, height)
    want_rgba, want_depth = oracle.splat(pm, vr, lit, cam, width, height)
    assert np.array_equal(depth, want_depth)
    assert np.array_equal(rgba, want_rgba)
    assert np.array_equal(rgba2, rgba) and np.array_equal(depth2, depth)
    assert (depth < 1.0).sum() > 100


_PIPELINED_SORT_CHECK = r"""
import sys
import numpy as np, torch
sys.path.insert(0, sys.argv[1])
from astro_gb300.radix_sort import RadixSort
rng = np.random.default_rng(5)
for n, bits in [(1, 64), (3071, 18), (3072, 18), (6144 * 3 + 5, 64), (1 << 20, 26), (5_000_001, 63)]:
    keys = rng.integers(0, 1 << min(bits, 63), n, dtype=np.uint64)
    keys[rng.integers(0, n, n // 3)] = keys[0]
    for off in (0, 1):  # 1: an input starting 8 bytes into a buffer (the fallback kernel)
        buf = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
        buf[off:off + n] = torch.from_numpy(keys.view(np.int64)).cuda()
        dk = buf[off:off + n]
        idx = torch.from_numpy(rng.permutation(n).astype(np.int32)).cuda()
        ok = torch.empty(n, dtype=torch.int64, device="cuda")
        oi = torch.empty(n, dtype=torch.int32, device="cuda")
        RadixSort(n, bits).sort(dk, idx, ok, oi, n)
        torch.cuda.synchronize()
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(ok.cpu().numpy().view(np.uint64), keys[order]), (n, bits, off)
        assert np.array_equal(oi.cpu().numpy(), idx.cpu().numpy()[order]), (n, bits, off)
print("ok")
"""


@pytest.mark.parametrize("variant_index", [7, 8, 9, 10, 11])
def test_sort_variants_match_stable_argsort(ag, tmp_path, variant_index):
    """The pipelined pass kernels (sort_variant 8 and 9) and the lean ones
    (10 to 12), each selected as the library default through
    ASTRO_SORT_VARIANT in a fresh process: whole and partial tiles, given
    indices, and unaligned inputs (the pipelined kernels fall back)."""
    import os
    import subprocess
    import sys

    script = tmp_path / "check.py"
    script.write_text(_PIPELINED_SORT_CHECK)
    env = dict(os.environ, ASTRO_SORT_VARIANT=str(variant_index))
    root = str(Path(__file__).resolve().parents[1])
    res = subprocess.run([sys.executable, str(script), root], capture_output=True, text=True,
                         env=env, timeout=600)
    assert res.returncode == 0 and "ok" in res.stdout, res.stderr[-2000:]


# ------------------------------------------------------ degenerate inputs --

def _degenerate(case):
    rng = np.random.default_rng(3)
    if case == "one":
        return np.array([[0.5, -0.25, 2.0]])
    if case == "two":
        return np.array([[0.0, 0.0, 0.0], [1e-3, 0.0, 0.0]])
    if case == "coincident":   # a zero-extent box: every key equal, one leaf
        return np.full((1000, 3), 0.25)
    if case == "line":         # two zero extents
        return np.stack([np.linspace(-1, 1, 3000), np.zeros(3000), np.zeros(3000)], axis=1)
    if case == "sheet":        # one zero extent, random in the plane
        xy = rng.uniform(-1, 1, (5000, 2))
        return np.concatenate([xy, np.zeros((5000, 1))], axis=1)
    raise KeyError(case)


@pytest.mark.parametrize("case", ["one", "two", "coincident", "line", "sheet"])
@pytest.mark.parametrize("form,far", [(0, 0.0), (1, 0.0), (0, 0.5), (1, 0.3)])
def test_degenerate_inputs_bit_exact(ag, oracle, case, form, far):
    """Boxes of zero extent in some or all axes, a single particle, and many
    coincident particles (one leaf), with and without far nodes (group
    boxes and displacements of zero length): same tree, forces and state as
    the CPU restatement, and finite everywhere."""
    L = ag.layouts
    pos = _degenerate(case)
    pm, vr = particles(L, pos, masses=np.full(len(pos), 1.0 / len(pos)))
    p = ag.default_params(L.PRESET_PHYSICAL, lbits=10, form=form, softening=0.01, far_ratio=far,
                          flags=WALKS["group"](L) | L.FLAG_IEEE_EXACT)
    out = run_gpu(ag, p, pm, vr, dt=1e-3, steps=2)
    pm_o, vr_o = pm.copy(), vr.copy()
    ref = oracle.phys_run(p, pm_o, vr_o, dt=1e-3, steps=2)
    assert_tree_equal(out, ref)
    assert np.array_equal(out["acc4"], ref["acc4"])
    assert np.isfinite(out["acc4"]).all() and np.isfinite(out["pm"]["position"]).all()
    assert np.array_equal(out["pm"], pm_o)
    n = len(pos)
    assert out["interactions"] == ref["interactions"] and out["interactions"] <= n * (n - 1) + n


def test_reference_coincident_bodies_bit_exact(ag, oracle):
    """REFERENCE preset: tree bodies sharing one position (one key, one
    leaf) and dust on top of them."""
    L = ag.layouts
    pos = np.concatenate([np.full((8, 3), 1e5), np.full((50, 3), 1e5)])
    pm, vr = particles(L, pos, masses=np.full(len(pos), 1000.0))
    ct = np.zeros(len(pos), L.COLOR_TYPE)
    ct["type"] = [1] * 8 + [2] * 50
    p = ag.default_params(L.PRESET_REFERENCE)
    out = run_gpu(ag, p, pm, vr, ct=ct, n_tree=8, dt=1.0 / 60, steps=2)
    pm_o, vr_o = pm.copy(), vr.copy()
    ref = oracle.ref_run(p, pm_o, vr_o, ct, n_tree=8, dt=1.0 / 60, steps=2, split_passes=64)
    assert_tree_equal(out, ref)
    assert np.array_equal(out["acc4"], ref["acc4"])
    assert np.array_equal(out["pm"], pm_o)


@pytest.mark.parametrize("weight,form", [(0.0, 0), (0.5, 1), (0.7, 0)])
def test_delta_weight_bit_exact(ag, oracle, weight, form):
    """The weight of the opening radius' delta term changes the walk; every
    weight must reproduce the CPU restatement bit for bit."""
    from astro_gb300 import ic

    L = ag.layouts
    p = ag.default_params(L.PRESET_PHYSICAL, lbits=12, form=form, open_delta_weight=weight,
                          softening=0.005, flags=WALKS["group"](L) | L.FLAG_IEEE_EXACT)
    pm, vr = ic.disk_bulge(16384, seed=1002)
    out = run_gpu(ag, p, pm, vr, dt=5e-4, steps=2)
    pm_o, vr_o = pm.copy(), vr.copy()
    ref = oracle.phys_run(p, pm_o, vr_o, dt=5e-4, steps=2)
    assert_tree_equal(out, ref)
    assert np.array_equal(out["acc4"], ref["acc4"])
    assert out["interactions"] == ref["interactions"] and out["node_visits"] == ref["node_visits"]


@pytest.mark.parametrize("ratio,form,walk,group_size,lbits", [
    (0.2, 0, "group", 32, 10), (0.3, 1, "group", 32, 12), (0.15, 0, "group-monopole", 32, 21),
    (0.25, 0, "group", 8, 10), (0.5, 1, "group", 1, 10), (0.4, 0, "group", 12, 6)])
def test_far_nodes_bit_exact(ag, oracle, ratio, form, walk, group_size, lbits):
    """Far nodes (one second-order expansion per group) in the exact form:
    the accelerations, the integrated state and every counter equal the
    CPU restatement's bit for bit."""
    from astro_gb300 import ic

    L = ag.layouts
    p = ag.default_params(L.PRESET_PHYSICAL, lbits=lbits, form=form, group_size=group_size,
                          far_ratio=ratio, flags=WALKS[walk](L) | L.FLAG_IEEE_EXACT)
    pm, vr = ic.plummer(16384, seed=1001)
    out = run_gpu(ag, p, pm, vr, dt=1e-3, steps=2)
    pm_o, vr_o = pm.copy(), vr.copy()
    ref = oracle.phys_run(p, pm_o, vr_o, dt=1e-3, steps=2)
    assert_tree_equal(out, ref)
    assert ref["far_nodes"] > 0
    for k in ("interactions", "node_visits", "far_nodes", "far_interactions"):
        assert out[k] == ref[k], k
    assert np.array_equal(out["acc4"], ref["acc4"])
    assert np.array_equal(out["pm"], pm_o) and np.array_equal(out["vr"], vr_o)


def test_far_nodes_batched_bit_exact(ag, oracle):
    from astro_gb300 import ic

    L = ag.layouts
    sizes = [1, 2, 31, 33, 1024, 5000, 64, 3, 4096, 777]
    parts = [ic.plummer(s, seed=1004, a=0.5 + 0.1 * k, system=k) for k, s in enumerate(sizes)]
    pm = np.concatenate([a for a, _ in parts])
    vr = np.concatenate([b for _, b in parts])
    p = ag.default_params(L.PRESET_PHYSICAL, far_ratio=0.25,
                          flags=WALKS["group"](L) | L.FLAG_IEEE_EXACT)
    out = run_gpu(ag, p, pm, vr, dt=1e-3, steps=2, sizes=sizes)
    pm_o, vr_o = pm.copy(), vr.copy()
    ref = oracle.phys_run(p, pm_o, vr_o, sizes=sizes, dt=1e-3, steps=2)
    assert_tree_equal(out, ref)
    assert out["far_nodes"] == ref["far_nodes"] > 0
    assert np.array_equal(out["acc4"], ref["acc4"])
    assert np.array_equal(out["pm"], pm_o)


@pytest.mark.parametrize("ratio,form,warps,group_size,walk", [
    (0.2, 0, 4, 32, "group"), (0.2, 1, 8, 32, "group"), (0.3, 0, 4, 12, "group"),
    (0.15, 1, 4, 4, "group"), (0.2, 0, 8, 32, "group-monopole")])
def test_far_nodes_fast_within_tolerance(ag, oracle, ratio, form, warps, group_size, walk):
    from astro_gb300 import ic

    L = ag.layouts
    p = ag.default_params(L.PRESET_PHYSICAL, flags=WALKS[walk](L), block_warps=warps,
                          softening=0.005, lbits=14, form=form, group_size=group_size,
                          far_ratio=ratio)
    pm, vr = ic.disk_bulge(32768, seed=1002)
    out = run_gpu(ag, p, pm, vr, dt=5e-4, steps=1)
    ref = oracle.phys_run(p, pm.copy(), vr.copy(), dt=5e-4, steps=1)
    assert_tree_equal(out, ref)
    ok, rel = acc_close(out["acc4"], ref["acc4"])
    assert ok.all(), f"{(~ok).sum()} particles outside tolerance, worst {rel.max():.3e}"
    assert ref["far_nodes"] > 0
    for k in ("interactions", "node_visits", "far_nodes", "far_interactions"):
        assert out[k] == ref[k], k


@pytest.mark.parametrize("form", [0, 1])
def test_build_per_layer_and_climbing_bit_exact(ag, oracle, form):
    """131,072 particles at lbits 12: the large bottom layers are aggregated
    one launch each and the small top layers in one climbing launch; the
    tree, the forces and the state must equal the restatement's."""
    from astro_gb300 import ic

    L = ag.layouts
    p = ag.default_params(L.PRESET_PHYSICAL, lbits=12, form=form, softening=0.005,
                          far_ratio=0.2, flags=WALKS["group"](L) | L.FLAG_IEEE_EXACT)
    pm, vr = ic.disk_bulge(131072, seed=1002)
    out = run_gpu(ag, p, pm, vr, dt=5e-4, steps=1)
    pm_o, vr_o = pm.copy(), vr.copy()
    ref = oracle.phys_run(p, pm_o, vr_o, dt=5e-4, steps=1)
    assert_tree_equal(out, ref)
    assert np.array_equal(out["acc4"], ref["acc4"])
    assert np.array_equal(out["pm"], pm_o) and np.array_equal(out["vr"], vr_o)


@pytest.mark.parametrize("case", ["plain", "far", "precision-far", "batched", "small-groups"])
def test_node_list_frontier_bit_exact(ag, oracle, case):
    """The group walk's other frontier form (a list of node indices instead
    of runs) visits the same nodes in the same order: every result equals
    the restatement's."""
    from astro_gb300 import ic

    L = ag.layouts
    kw = dict(lbits=10, walk_frontier=1, flags=WALKS["group"](L) | L.FLAG_IEEE_EXACT)
    sizes = None
    if case == "far":
        kw.update(far_ratio=0.3)
    elif case == "precision-far":
        kw.update(far_ratio=0.2, form=L.FORM_PRECISION)
    elif case == "small-groups":
        kw.update(group_size=5)
    if case == "batched":
        sizes = [1, 2, 31, 33, 1024, 5000, 64, 3, 4096, 777]
        parts = [ic.plummer(s_, seed=1004, a=0.5 + 0.1 * k, system=k) for k, s_ in enumerate(sizes)]
        pm = np.concatenate([a_ for a_, _ in parts])
        vr = np.concatenate([b_ for _, b_ in parts])
        kw.update(far_ratio=0.25)
    else:
        pm, vr = ic.plummer(16384, seed=1001)
    p = ag.default_params(L.PRESET_PHYSICAL, **kw)
    out = run_gpu(ag, p, pm, vr, dt=1e-3, steps=2, sizes=sizes)
    pm_o, vr_o = pm.copy(), vr.copy()
    ref = oracle.phys_run(p, pm_o, vr_o, sizes=sizes, dt=1e-3, steps=2)
    assert_tree_equal(out, ref)
    for k in ("interactions", "node_visits", "far_nodes", "far_interactions"):
        assert out[k] == ref[k], k
    assert np.array_equal(out["acc4"], ref["acc4"])
    assert np.array_equal(out["pm"], pm_o) and np.array_equal(out["vr"], vr_o)
