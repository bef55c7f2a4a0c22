"""Seeded random configurations of the PHYSICAL preset in the IEEE-exact
form: size, depth, group size, bucket, far ratio, frontier form, precision,
batching and the distribution all vary; every result must equal the CPU
restatement's bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = 24


@pytest.fixture(scope="module")
def ag(native):
    return native


def _config(k):
    rng = np.random.default_rng(9000 + k)
    cfg = dict(
        n=int(rng.choice([1, 2, 7, 33, 500, 4097, 12000, 30000])),
        lbits=int(rng.integers(1, 22)),
        group_size=int(rng.integers(1, 33)),
        bucket=int(rng.choice([0, 1, 8, 16, 64])),
        far_ratio=float(rng.choice([0.0, 0.1, 0.25, 0.5])),
        walk_frontier=int(rng.integers(0, 2)),
        form=int(rng.integers(0, 2)),
        quad=bool(rng.integers(0, 2)),
        delta=bool(rng.integers(0, 2)),
        dist=str(rng.choice(["plummer", "cube", "disk"])),
        nsys=int(rng.choice([1, 1, 3])),
    )
    return cfg


def _particles(L, ic, cfg):
    n, nsys = cfg["n"], cfg["nsys"]
    sizes = None
    if nsys > 1 and n >= 3:
        base = n // nsys
        sizes = [base] * (nsys - 1) + [n - base * (nsys - 1)]
    parts = []
    for s, m in enumerate(sizes or [n]):
        if cfg["dist"] == "plummer":
            parts.append(ic.plummer(m, seed=17, system=s))
        elif cfg["dist"] == "cube":
            parts.append(ic.uniform_cube(m, seed=17 + s))
        else:
            parts.append(ic.disk_bulge(max(m, 2), seed=17 + s) if m >= 2 else ic.plummer(m, seed=17, system=s))
    pm = np.concatenate([a for a, _ in parts])[:n]
    vr = np.concatenate([b for _, b in parts])[:n]
    if sizes is not None and sum(sizes) != len(pm):
        sizes = None
    return pm, vr, sizes


def _large_groups(cfg, k):
    """Groups of 33 to 64 particles (two per lane; the chunks of a leaf
    that holds more share one walk, and with far nodes their sums are
    formed once per walk by their own kernel)."""
    rng = np.random.default_rng(9700 + k)
    cfg.update(group_size=int(rng.integers(33, 65)), far_ratio=float(rng.choice([0.0, 0.25, 0.5])),
               n=int(rng.choice([7, 500, 4097, 12000, 30000])), lbits=int(rng.integers(1, 6)))
    return cfg


@pytest.mark.parametrize("k", range(CASES + 12))
def test_random_configuration_bit_exact(ag, oracle, k):
    from astro_gb300 import ic
    from test_gpu_parity import assert_tree_equal, run_gpu

    L = ag.layouts
    cfg = _config(k) if k < CASES else _large_groups(_config(k), k)
    flags = L.FLAG_IEEE_EXACT | (L.FLAG_QUADRUPOLE if cfg["quad"] else 0) | (
        L.FLAG_OPEN_DELTA if cfg["delta"] else 0)
    pm, vr, sizes = _particles(L, ic, cfg)
    nsys = len(sizes) if sizes else 1
    if 3 * cfg["lbits"] + ((nsys - 1).bit_length() if nsys > 1 else 0) > 64:
        cfg["lbits"] = 20
    p = ag.default_params(L.PRESET_PHYSICAL, lbits=cfg["lbits"], group_size=cfg["group_size"],
                          bucket=cfg["bucket"], far_ratio=cfg["far_ratio"],
                          walk_frontier=cfg["walk_frontier"], form=cfg["form"], softening=0.01,
                          flags=flags)
    out = run_gpu(ag, p, pm, vr, dt=1e-3, steps=2, sizes=sizes)
    pm_o, vr_o = pm.copy(), vr.copy()
    ref = oracle.phys_run(p, pm_o, vr_o, sizes=sizes, dt=1e-3, steps=2)
    assert_tree_equal(out, ref)
    for key in ("interactions", "node_visits", "far_nodes", "far_interactions"):
        assert out[key] == ref[key], (cfg, key)
    assert np.array_equal(out["acc4"], ref["acc4"]), cfg
    assert np.array_equal(out["pm"], pm_o) and np.array_equal(out["vr"], vr_o), cfg


def _ref_config(k):
    rng = np.random.default_rng(9500 + k)
    return dict(n_stars=int(rng.integers(0, 6)), n_planets=int(rng.choice([0, 1, 50, 200, 700])),
                n_dust=int(rng.choice([0, 1, 100, 3000])), lbits=int(rng.integers(1, 11)),
                steps=int(rng.integers(1, 4)), lights=int(rng.integers(0, 6)))


@pytest.mark.parametrize("k", range(12))
def test_random_reference_scene_bit_exact(ag, oracle, k):
    """The REFERENCE preset over random scene sizes, depths, step counts and
    light counts: keys, tree, forces, lit colours and the integrated state
    equal the reference transcription's."""
    from astro_gb300 import ic
    from test_gpu_parity import assert_tree_equal, run_gpu

    L = ag.layouts
    cfg = _ref_config(k)
    n_tree = cfg["n_stars"] + cfg["n_planets"]
    if n_tree == 0:
        cfg["n_planets"] = n_tree = 1
    pm, vr, ct = ic.reference_scene(cfg["n_stars"], cfg["n_planets"], cfg["n_dust"], seed=31 + k)
    p = ag.default_params(L.PRESET_REFERENCE, lbits=cfg["lbits"],
                          light_sources=min(cfg["lights"], cfg["n_stars"] + cfg["n_planets"]))
    out = run_gpu(ag, p, pm, vr, ct, n_tree=n_tree, dt=1.0 / 60, steps=cfg["steps"])
    pm_o, vr_o, ct_o = pm.copy(), vr.copy(), ct.copy()
    ref = oracle.ref_run(p, pm_o, vr_o, ct_o, n_tree=n_tree, dt=1.0 / 60, steps=cfg["steps"],
                         split_passes=64)
    assert_tree_equal(out, ref)
    assert np.array_equal(out["acc4"], ref["acc4"]), cfg
    assert np.array_equal(out["pm"], pm_o) and np.array_equal(out["vr"], vr_o), cfg


@pytest.mark.parametrize("k", range(16 + 8))
def test_random_configuration_fast_within_tolerance(ag, oracle, k):
    """The fast form (rsqrt, FMAs, replicated small groups, factored far-node
    coefficients, groups of up to 64 in packed pairs) over random
    configurations: the same walk (identical counts) and accelerations
    within the fast path's tolerance."""
    from astro_gb300 import ic
    from test_gpu_parity import acc_close, assert_tree_equal, run_gpu

    L = ag.layouts
    cfg = _config(100 + k) if k < 16 else _large_groups(_config(100 + k), 100 + k)
    cfg["n"] = max(cfg["n"], 500)
    flags = (L.FLAG_QUADRUPOLE if cfg["quad"] else 0) | (L.FLAG_OPEN_DELTA if cfg["delta"] else 0)
    pm, vr, sizes = _particles(L, ic, cfg)
    nsys = len(sizes) if sizes else 1
    if 3 * cfg["lbits"] + ((nsys - 1).bit_length() if nsys > 1 else 0) > 64:
        cfg["lbits"] = 20
    p = ag.default_params(L.PRESET_PHYSICAL, lbits=cfg["lbits"], group_size=cfg["group_size"],
                          bucket=cfg["bucket"], far_ratio=cfg["far_ratio"],
                          walk_frontier=cfg["walk_frontier"], form=cfg["form"], softening=0.01,
                          block_warps=8 if k % 2 else 4, flags=flags)
    out = run_gpu(ag, p, pm, vr, dt=1e-3, steps=1, sizes=sizes)
    ref = oracle.phys_run(p, pm.copy(), vr.copy(), sizes=sizes, dt=1e-3, steps=1)
    assert_tree_equal(out, ref)
    for key in ("interactions", "node_visits", "far_nodes", "far_interactions"):
        assert out[key] == ref[key], (cfg, key)
    ok, rel = acc_close(out["acc4"], ref["acc4"])
    assert ok.all(), f"{cfg}: {(~ok).sum()} particles outside tolerance, worst {rel.max():.3e}"


# Full groups (more than 16 particles, so no replication) in the precision
# form's fast path, which evaluates cells and leaf particles two at a time in
# packed FP32 pairs; the list lengths of a flush are odd and even alike.
PAIR_CASES = [
    dict(n=4097, group_size=32, far_ratio=0.0, walk_frontier=0, nsys=1, dist="plummer"),
    dict(n=20000, group_size=24, far_ratio=0.3, walk_frontier=1, nsys=1, dist="disk"),
    dict(n=6001, group_size=32, far_ratio=0.15, walk_frontier=0, nsys=3, dist="cube"),
    dict(n=12345, group_size=17, far_ratio=0.0, walk_frontier=1, nsys=1, dist="cube"),
]


@pytest.mark.parametrize("k", range(len(PAIR_CASES)))
def test_precision_pairs_within_tolerance(ag, oracle, k):
    """Precision form, fast path, quadrupoles and the δ opening: the same
    tree and counts as the CPU restatement, accelerations within the fast
    path's tolerance."""
    from astro_gb300 import ic
    from test_gpu_parity import acc_close, assert_tree_equal, run_gpu

    L = ag.layouts
    cfg = dict(lbits=10, bucket=8, quad=True, delta=True, form=L.FORM_PRECISION)
    cfg.update(PAIR_CASES[k])
    flags = L.FLAG_QUADRUPOLE | L.FLAG_OPEN_DELTA
    pm, vr, sizes = _particles(L, ic, cfg)
    p = ag.default_params(L.PRESET_PHYSICAL, lbits=cfg["lbits"], group_size=cfg["group_size"],
                          bucket=cfg["bucket"], far_ratio=cfg["far_ratio"],
                          walk_frontier=cfg["walk_frontier"], form=cfg["form"], softening=0.01,
                          block_warps=8 if k % 2 else 4, flags=flags)
    out = run_gpu(ag, p, pm, vr, dt=1e-3, steps=1, sizes=sizes)
    ref = oracle.phys_run(p, pm.copy(), vr.copy(), sizes=sizes, dt=1e-3, steps=1)
    assert_tree_equal(out, ref)
    for key in ("interactions", "node_visits", "far_nodes", "far_interactions"):
        assert out[key] == ref[key], (cfg, key)
    ok, rel = acc_close(out["acc4"], ref["acc4"])
    assert ok.all(), f"{cfg}: {(~ok).sum()} particles outside tolerance, worst {rel.max():.3e}"
