"""Known-answer tests of the CPU restatement (oracle/) against the hand-derived
golden vectors in tests/golden (the reference ships none of its own)."""
import json
from pathlib import Path

import numpy as np
import pytest

from astro_gb300 import layouts as L

GOLDEN = Path(__file__).resolve().parent / "golden"


def load(name):
    return json.loads((GOLDEN / f"{name}.json").read_text())


def ref_params(**kw):
    """REFERENCE defaults without loading the CUDA library."""
    p = L.Params(preset=L.PRESET_REFERENCE, form=0, lbits=6, flags=0, theta=0.7, g=1e11,
                 softening=0.01, leaf_min_dist2=50.0, force_clamp=1e5, quant_offset=1e6,
                 damping=0.9995, bucket=0, block_warps=0, open_delta_weight=1.0)
    p.type_accel_scale[0], p.type_accel_scale[1], p.type_accel_scale[2] = 5.0, 5.0, 1.0
    return p.replace(**kw) if kw else p


def phys_params(**kw):
    p = L.Params(preset=L.PRESET_PHYSICAL, form=0, lbits=6,
                 flags=L.FLAG_OPEN_DELTA | L.FLAG_QUADRUPOLE, theta=0.7, g=1.0,
                 softening=0.01, leaf_min_dist2=0.0, force_clamp=1e5, quant_offset=0.0,
                 damping=1.0, bucket=16, block_warps=0, open_delta_weight=1.0)
    for i in range(3):
        p.type_accel_scale[i] = 1.0
    return p.replace(**kw) if kw else p


def particles(pos, masses=None):
    n = len(pos)
    pm, vr = L.empty_particles(n)
    pm["position"] = np.asarray(pos, np.float32)
    pm["mass"] = 1.0 if masses is None else np.asarray(masses, np.float32)
    return pm, vr


def test_interleave_bit_placement(oracle):
    for i in range(21):
        assert oracle.interleave(1 << i, 0, 0) == 1 << (3 * i)
        assert oracle.interleave(0, 1 << i, 0) == 1 << (3 * i + 1)
        assert oracle.interleave(0, 0, 1 << i) == 1 << (3 * i + 2)
    # Bits above 21 are masked off (MortonCode.metal:9-11).
    assert oracle.interleave(1 << 21, 0, 0) == 0


def test_morton_golden(oracle):
    g = load("morton")
    pos = [c["pos"] for c in g["cases"]]
    pm, _ = particles(pos)
    codes = oracle.morton_codes(pm, g["lbits"], g["offset"])
    assert [int(c) for c in codes] == [c["key"] for c in g["cases"]]


def test_exclusive_scan_beyond_reference_limit(oracle):
    # The reference's two-level scan stops at 1,048,576 values; the
    # restatement lifts the limit without changing smaller results.
    rng = np.random.default_rng(3)
    for n in [1, 2, 1023, 1024, 1025, 1 << 20, (1 << 20) + 7, 3_000_001]:
        v = rng.integers(0, 3, n).astype(np.uint32)
        want = np.concatenate([[0], np.cumsum(v, dtype=np.uint64)[:-1]]).astype(np.uint32)
        assert np.array_equal(oracle.exclusive_scan(v), want), n


def test_split_sort_golden_and_stability(oracle):
    g = load("sort")
    keys, perm = oracle.split_sort(np.array(g["keys"], np.uint64), passes=64)
    assert [int(i) for i in perm] == g["perm"]
    rng = np.random.default_rng(5)
    k = rng.integers(0, 1 << 18, 50000).astype(np.uint64)
    k[::7] = k[3]  # many duplicates
    ok, oi = oracle.split_sort(k, passes=64)
    want = np.argsort(k, kind="stable")
    assert np.array_equal(oi, want) and np.array_equal(ok, k[want])
    # Skipping the constant-zero high bits gives the identical permutation.
    ok18, oi18 = oracle.split_sort(k, passes=18)
    assert np.array_equal(oi18, oi)


def test_layer_layout_closed_form(oracle):
    sizes, offsets, cap = oracle.layer_layout(205, 6)
    # Renderer.swift:373-386 with octreeCount = 205.
    assert list(sizes) == [205, 205, 205, 205, 64, 8, 1]
    assert list(offsets) == [0, 205, 410, 615, 820, 884, 892]
    assert cap == 893
    sizes, offsets, cap = oracle.layer_layout(1 << 24, 21)
    assert sizes[0] == 1 << 24 and sizes[-1] == 1 and sizes[13] == 1 << 24 and sizes[14] == 1 << 21


def test_octant_tree_golden(oracle):
    g = load("octants")
    pm, vr = particles(g["positions"])
    out = oracle.ref_run(ref_params(), pm, vr, dt=0.0, steps=1)
    assert [int(k) for k in out["codes"]] == g["keys"]
    assert [int(i) for i in out["sorted_indices"]] == g["sorted_indices"]
    assert list(out["layer_counts"]) == g["layer_counts"]
    assert list(out["layer_sizes"]) == g["layer_sizes"]
    assert list(out["layer_offsets"]) == g["layer_offsets"]
    root = out["nodes"][g["root"]]
    assert list(root["children"]) == g["root_children"]
    assert root["totalMass"] == g["root_mass"]
    assert np.allclose(root["centerOfMass"], g["root_com"], rtol=0, atol=0.5)
    assert root["layer"] == 6
    # Every layer-1..5 node has exactly one child.
    for node in out["nodes"][8:48]:
        assert node["children"][0] != L.INVALID_CHILD and node["children"][1] == L.INVALID_CHILD
    for leaf in out["nodes"][:8]:
        assert all(c == L.INVALID_CHILD for c in leaf["children"])


@pytest.mark.parametrize("case", range(4))
def test_two_body_golden(oracle, case):
    g = load("two_body")
    c = g["cases"][case]
    pm, vr = particles([(c["x0"], 0, 0), (c["x0"] + c["d"], 0, 0)], [c["m"], c["m"]])
    out = oracle.ref_run(ref_params(), pm, vr, dt=0.0, steps=1)
    acc = out["acc4"]
    assert acc[0, 0] == pytest.approx(c["fx0"], rel=1e-5, abs=0)
    assert acc[1, 0] == pytest.approx(c["fx1"], rel=1e-5, abs=0)
    assert acc[0, 1] == 0 and acc[0, 2] == 0


def test_last_leaf_quirk_reference_and_fix(oracle):
    g = load("last_leaf")
    pm, vr = particles(g["positions"], g["masses"])
    out = oracle.ref_run(ref_params(), pm.copy(), vr.copy(), dt=0.0, steps=1)
    assert list(out["layer_counts"][:1]) == [2]
    leaves = out["nodes"][:2]
    assert list(leaves["totalMass"]) == g["reference_leaf_mass"]
    assert np.array_equal(leaves["centerOfMass"], np.array(g["reference_leaf_com"], np.float32))
    out = oracle.phys_run(phys_params(), pm.copy(), vr.copy(), dt=0.0, steps=1)
    leaves = out["nodes"][:2]
    assert list(leaves["totalMass"]) == g["fixed_leaf_mass"]


def test_reference_integrator(oracle):
    # updateSpheres (BarnesHut.metal:169-196): a = F * {5,5,1}[type];
    # v = 0.9995 v + a dt; x += v dt. A lone body feels no force.
    pm, vr = particles([(10.0, 20.0, 30.0)])
    vr["velocity"] = [[1.0, 2.0, 3.0]]
    oracle.ref_run(ref_params(), pm, vr, dt=0.5, steps=1)
    v = np.float32(0.9995) * np.array([1.0, 2.0, 3.0], np.float32)
    assert np.array_equal(vr["velocity"][0], v)
    assert np.array_equal(pm["position"][0], np.array([10, 20, 30], np.float32) + v * np.float32(0.5))


def test_physical_tiny_theta_is_direct_sum(oracle, native):
    # With theta -> 0 nothing is accepted: every opened leaf is summed
    # particle by particle, which is the softened direct sum.
    from astro_gb300 import ic  # host generator, no GPU involved

    pm, vr = ic.plummer(2048, seed=11)
    p = phys_params(theta=1e-6, softening=0.05)
    out = oracle.phys_run(p, pm.copy(), vr.copy(), dt=0.0, steps=1)
    samples = np.arange(0, 2048, 7)
    direct = oracle.direct_accel(pm, samples, g=1.0, eps=0.05)
    got = out["acc4"][samples, :3].astype(np.float64)
    err = np.linalg.norm(got - direct, axis=1) / np.linalg.norm(direct, axis=1)
    assert np.max(err) < 1e-4
    assert out["interactions"] == 2048 * 2047


@pytest.mark.parametrize("flags,median_max", [
    (L.FLAG_PER_PARTICLE, 5e-3),                                      # the reference's walk
    (L.FLAG_PER_PARTICLE | L.FLAG_OPEN_DELTA | L.FLAG_QUADRUPOLE, 1.5e-3),
    (L.FLAG_OPEN_DELTA | L.FLAG_QUADRUPOLE, 1e-3),                   # group walk (default)
])
def test_physical_error_against_direct_sum(oracle, native, flags, median_max):
    from astro_gb300 import ic

    pm, vr = ic.plummer(8192, seed=1001)
    p = phys_params(theta=0.7, lbits=21, flags=flags)
    out = oracle.phys_run(p, pm.copy(), vr.copy(), dt=0.0, steps=1)
    samples = np.arange(0, 8192, 13)
    direct = oracle.direct_accel(pm, samples, g=1.0, eps=float(np.float32(0.01)))
    got = out["acc4"][samples, :3].astype(np.float64)
    err = np.linalg.norm(got - direct, axis=1) / np.linalg.norm(direct, axis=1)
    assert np.median(err) < median_max and np.percentile(err, 99) < 5e-2


def test_physical_batched_equals_separate(oracle, native):
    from astro_gb300 import ic

    pm1, vr1 = ic.plummer(700, seed=3, system=0)
    pm2, vr2 = ic.plummer(1300, seed=3, a=2.0, system=1)
    pm = np.concatenate([pm1, pm2])
    vr = np.concatenate([vr1, vr2])
    p = phys_params()
    both = oracle.phys_run(p, pm.copy(), vr.copy(), sizes=[700, 1300], dt=1e-3, steps=2)
    a = oracle.phys_run(p, pm1.copy(), vr1.copy(), dt=1e-3, steps=2)
    b = oracle.phys_run(p, pm2.copy(), vr2.copy(), dt=1e-3, steps=2)
    assert np.array_equal(both["acc4"][:700], a["acc4"])
    assert np.array_equal(both["acc4"][700:], b["acc4"])


def test_group_walk_covers_every_particle_once(oracle, native):
    # The group list partitions the particles: with theta -> 0 every particle
    # interacts with every other exactly once, whatever the group layout.
    from astro_gb300 import ic

    for lbits, n, gsize in [(6, 3000, 0), (21, 3000, 0), (3, 500, 0), (10, 2000, 1),
                            (10, 2000, 7), (6, 3000, 16)]:
        pm, vr = ic.disk_bulge(n, seed=4)
        p = phys_params(theta=1e-6, lbits=lbits, group_size=gsize)
        out = oracle.phys_run(p, pm.copy(), vr.copy(), dt=0.0)
        assert out["interactions"] == n * (n - 1)


def test_smaller_groups_test_more_nodes(oracle, native):
    # Smaller groups have tighter boxes: fewer interactions and node tests
    # per particle (but more walks); the same tree and nearly the same
    # accelerations.
    from astro_gb300 import ic

    pm, vr = ic.plummer(8192, seed=1001)
    runs = {g: oracle.phys_run(phys_params(lbits=14, group_size=g), pm.copy(), vr.copy(), dt=0.0)
            for g in (8, 32)}
    assert runs[8]["interactions"] < runs[32]["interactions"]
    assert runs[8]["node_visits"] < runs[32]["node_visits"]
    assert np.array_equal(runs[8]["sorted_codes"], runs[32]["sorted_codes"])
    a8, a32 = runs[8]["acc4"][:, :3], runs[32]["acc4"][:, :3]
    rel = np.linalg.norm(a8 - a32, axis=1) / np.linalg.norm(a32, axis=1)
    assert np.median(rel) < 2e-3


def test_precision_form_runs_and_tracks_plain(oracle, native):
    from astro_gb300 import ic

    pm, vr = ic.plummer(4096, seed=9)
    plain = oracle.phys_run(phys_params(), pm.copy(), vr.copy(), dt=1e-3, steps=3)
    prec = oracle.phys_run(phys_params(form=L.FORM_PRECISION), pm.copy(), vr.copy(), dt=1e-3,
                           steps=3, want_pos64=True)
    d = np.abs(plain["acc4"] - prec["acc4"]).max() / np.abs(plain["acc4"]).max()
    assert d < 1e-3
    assert prec["pos64"].shape == (4096, 3)


def test_lighting_known_answers(oracle):
    # One star at the origin (rgb 1, 0.5, 0.25); a planet at the attenuation
    # distance 4e5 gets exactly the star's colour; dust at 8e5 a quarter of it
    # and alpha min(max channel, 0.25); a second star is left alone.
    pm, _ = particles([[0, 0, 0], [4e5, 0, 0], [0, 8e5, 0], [0, 0, 3e5]])
    ct = np.zeros(4, L.COLOR_TYPE)
    ct["type"] = [0, 1, 2, 0]
    ct["color"][0] = [1.0, 0.5, 0.25, 1.0]
    ct["color"][3] = [0.1, 0.2, 0.3, 1.0]
    out = oracle.lighting(pm, ct, num_stars=1)
    assert out["color"][1].tolist() == [1.0, 0.5, 0.25, 1.0]
    assert out["color"][2].tolist() == [0.25, 0.125, 0.0625, 0.25]
    assert out["color"][3].tolist() == pytest.approx([0.1, 0.2, 0.3, 1.0])
    assert np.array_equal(out["color"][0], ct["color"][0])
    # The lights are the first num_stars particles, read before the pass: a
    # planet among them lights with its colour from before (zero here).
    two = oracle.lighting(pm, ct, num_stars=2)
    assert two["color"][2].tolist() == [0.25, 0.125, 0.0625, 0.25]
    ct_b = ct.copy()
    ct_b["color"][1] = [0.5, 0.5, 0.5, 1.0]
    three = oracle.lighting(pm, ct_b, num_stars=2)
    assert three["color"][2][0] == pytest.approx(0.25 + 0.5 / (np.hypot(4e5, 8e5) / 4e5) ** 2)
    # A planet on top of a light saturates at 1 / (1e-9)^2.
    pm2, _ = particles([[0, 0, 0], [0, 0, 0]])
    ct2 = np.zeros(2, L.COLOR_TYPE)
    ct2["type"] = [0, 1]
    ct2["color"][0] = [1.0, 0, 0, 1]
    assert oracle.lighting(pm2, ct2, 1)["color"][1][0] == np.float32(1.0 / np.float32(1e-9) ** 2)


def _flat_camera():
    # view = identity, projection = identity: clip = (x - cam, 1), so window
    # coordinates follow directly from the positions.
    from astro_gb300.render import Camera

    eye = np.eye(4, dtype=np.float32).reshape(16)
    return Camera(eye.copy(), eye.copy(), np.zeros(3, np.float32))


def test_splat_half_rounding_matches_ieee_binary16(oracle):
    # A one-pixel image whose only fragment is an opaque disc of colour x
    # returns round_to_half(x): compare with numpy's float16 conversion.
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.normal(0, 1, 200), rng.normal(0, 1e4, 50), [6.1e-5, 5.9e-8, 65519.0,
                         65520.0, 0.1, 1 / 255]]).astype(np.float32)
    pm, vr = particles([[0.0, 0.0, 0.5]])
    vr["radius"] = 4.0
    ct = np.zeros(1, L.COLOR_TYPE)
    ct["type"] = 0
    for x in xs:
        ct["color"][0] = [x, -x, x / 3, 1.0]
        rgba, _ = oracle.splat(pm, vr, ct, _flat_camera(), 1, 1)
        with np.errstate(over="ignore"):
            want = np.array([x, -x, np.float32(x) / np.float32(3)], np.float32).astype(np.float16)
        assert np.array_equal(rgba[0, 0, :3], want.astype(np.float32)), x


def test_splat_points_discs_depth_and_blending(oracle):
    from astro_gb300.render import Camera

    cam = _flat_camera()
    W = H = 8
    # A dust point of size 2 at the image centre covers the 2 x 2 pixels
    # around it and blends over the clear colour.
    pm, vr = particles([[0.0, 0.0, 0.5]])
    vr["radius"] = 2.0
    ct = np.zeros(1, L.COLOR_TYPE)
    ct["type"] = 2
    ct["color"][0] = [1.0, 0.5, 0.25, 0.25]
    clear = np.array([0.0, 0.0, 1.0 / 255.0, 1.0], np.float32)
    rgba, depth = oracle.splat(pm, vr, ct, cam, W, H, clear)
    hit = depth < 1.0
    assert hit.sum() == 4 and hit[3:5, 3:5].all()
    c16 = clear.astype(np.float16).astype(np.float32)
    a = np.float32(0.25)
    want_r = np.float16(np.float32(1.0) * a + c16[0] * (np.float32(1) - a)).astype(np.float32)
    want_b = np.float16(np.float32(0.25) * a + c16[2] * (np.float32(1) - a)).astype(np.float32)
    assert rgba[3, 3, 0] == want_r and rgba[3, 3, 2] == want_b
    assert np.array_equal(rgba[0, 0], c16) and depth[0, 0] == 1.0
    # Two opaque discs: the nearer one wins whatever the draw order; a disc
    # of radius r (world r/2, H/2 pixels per unit) covers centres within r px.
    pm, vr = particles([[0.0, 0.0, 0.8], [0.0, 0.0, 0.3]])
    vr["radius"] = [1.0, 0.5]      # discs of 2 px and 1 px: (radius / 2) * (H / 2)
    ct = np.zeros(2, L.COLOR_TYPE)
    ct["type"] = [0, 1]
    ct["color"] = [[1, 0, 0, 1], [0, 1, 0, 1]]
    rgba, depth = oracle.splat(pm, vr, ct, cam, W, H)
    near = depth == np.float32(0.3)
    far = depth == np.float32(0.8)
    # The 2 px disc covers the 12 centres within distance 2 of (4, 4); the
    # 1 px disc in front of it covers the middle 4.
    assert near.sum() == 4 and far.sum() == 8
    assert (rgba[near][:, 1] == 1.0).all() and (rgba[far][:, 0] == 1.0).all()
    rev = oracle.splat(pm[::-1].copy(), vr[::-1].copy(), ct[::-1].copy(), cam, W, H)
    assert np.array_equal(rev[0], rgba) and np.array_equal(rev[1], depth)
    # Behind the camera (w <= 0) or beyond the far plane nothing is drawn.
    pm, vr = particles([[0.0, 0.0, 1.5]])
    vr["radius"] = 2.0
    rgba, depth = oracle.splat(pm, vr, ct[:1], cam, W, H)
    assert (depth == 1.0).all()


def test_delta_weight_zero_is_the_plain_opening_radius(oracle, native):
    # w = 0 turns size/theta + w delta into size/theta exactly: the same walk
    # and forces as without the delta flag; a larger w opens more nodes.
    from astro_gb300 import ic

    pm, vr = ic.disk_bulge(6000, seed=2)
    no_delta = oracle.phys_run(phys_params(flags=L.FLAG_QUADRUPOLE), pm.copy(), vr.copy(), dt=0.0)
    w0 = oracle.phys_run(phys_params(open_delta_weight=0.0), pm.copy(), vr.copy(), dt=0.0)
    w1 = oracle.phys_run(phys_params(), pm.copy(), vr.copy(), dt=0.0)
    assert np.array_equal(no_delta["acc4"], w0["acc4"])
    assert no_delta["interactions"] == w0["interactions"] < w1["interactions"]


def _field64(D, m, Q, eps2):
    """FP64 field of a node with quadrupole at displacement D (as the walk's terms)."""
    r2 = D @ D + eps2
    r = np.sqrt(r2)
    qd = Q @ D
    return m * D / r**3 + 2.5 * (D @ qd) * D / r**7 - qd / r**5


def test_far_expansion_coefficients_are_the_taylor_series(oracle):
    # The 19 coefficients of a far node are its field and that field's first
    # and second derivatives at D = com - centre (checked against central
    # differences of the FP64 field), and the expansion reproduces the field
    # at an offset rho to third order in |rho| / |D|.
    rng = np.random.default_rng(7)
    xs = rng.uniform(-0.5, 0.5, (40, 3))
    ms = rng.uniform(0.5, 1.5, 40)
    com = (ms[:, None] * xs).sum(0) / ms.sum()
    d = xs - com
    Q = sum(m * (3 * np.outer(v, v) - v @ v * np.eye(3)) for v, m in zip(d, ms))
    q5 = np.array([Q[0, 0], Q[1, 1], Q[0, 1], Q[0, 2], Q[1, 2]], np.float32)
    Q = np.array([[q5[0], q5[2], q5[3]], [q5[2], q5[1], q5[4]], [q5[3], q5[4], -(q5[0] + q5[1])]],
                 np.float64)
    eps = 0.01
    p = phys_params(softening=eps, g=2.0)
    gc = np.array([0.3, -0.2, 0.1], np.float32)
    cm4 = np.array([8.0, -5.0, 3.0, ms.sum()], np.float32)
    D = cm4[:3].astype(np.float64) - gc
    m = float(cm4[3])
    co, _ = oracle.far_expand(p, cm4, q5, gc, np.zeros(3))
    eps2 = float(np.float32(eps) * np.float32(eps))
    a = _field64(D, m, Q, eps2)
    h = 1e-4
    J = np.zeros((3, 3))
    H = np.zeros((3, 3, 3))
    for j in range(3):
        e = np.zeros(3)
        e[j] = h
        J[:, j] = (_field64(D + e, m, Q, eps2) - _field64(D - e, m, Q, eps2)) / (2 * h)
        for k in range(3):
            f = np.zeros(3)
            f[k] = h
            H[:, j, k] = (_field64(D + e + f, m, Q, eps2) - _field64(D + e - f, m, Q, eps2)
                          - _field64(D - e + f, m, Q, eps2) + _field64(D - e - f, m, Q, eps2)) / (4 * h * h)
    jj = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]
    hh = [(0, 0, 0), (1, 1, 1), (2, 2, 2), (0, 0, 1), (0, 0, 2), (0, 1, 1), (1, 1, 2), (0, 2, 2),
          (1, 2, 2), (0, 1, 2)]
    want = np.concatenate([a, [J[i, j] for i, j in jj], [H[i, j, k] for i, j, k in hh]])
    scale = np.concatenate([np.full(3, np.abs(a).max()), np.full(6, np.abs(J).max()),
                            np.full(10, np.abs(H).max())])
    assert np.all(np.abs(co - want) <= 1e-4 * scale), np.abs(co - want) / scale
    # The expansion at offsets up to 10% of |D|: error ~ (|rho|/|D|)^3.
    for frac in (0.02, 0.05, 0.1):
        rho = rng.normal(size=3)
        rho *= frac * np.linalg.norm(D) / np.linalg.norm(rho)
        _, acc = oracle.far_expand(p, cm4, q5, gc, rho.astype(np.float32))
        exact = 2.0 * _field64(D - rho.astype(np.float32), m, Q, eps2)
        rel = np.linalg.norm(acc - exact) / np.linalg.norm(exact)
        assert rel < 2.0 * frac**3 + 1e-5, (frac, rel)


def test_far_nodes_keep_the_walk_and_the_accuracy(oracle, native):
    # far_ratio changes how accepted nodes are summed, never which: the
    # interaction and visit counts stay, the far counts grow with the ratio,
    # and the accelerations stay within the expansion's third-order error
    # (the error against the FP64 direct sum barely moves).
    from astro_gb300 import ic

    pm, vr = ic.plummer(16384, seed=1001)
    samples = np.random.default_rng(0).choice(len(pm), 256, replace=False)
    ref = oracle.direct_accel(pm, samples, g=1.0, eps=0.01)
    runs = {r: oracle.phys_run(phys_params(lbits=10, far_ratio=r), pm.copy(), vr.copy(), dt=0.0)
            for r in (0.0, 0.1, 0.2)}
    base = runs[0.0]
    assert base["far_nodes"] == 0 and base["far_interactions"] == 0
    errs = {}
    for r, out in runs.items():
        assert out["interactions"] == base["interactions"]
        assert out["node_visits"] == base["node_visits"]
        acc = out["acc4"].reshape(-1, 4)[samples, :3].astype(np.float64)
        errs[r] = np.median(np.linalg.norm(acc - ref, axis=1) / np.linalg.norm(ref, axis=1))
    assert 0 < runs[0.1]["far_interactions"] < runs[0.2]["far_interactions"] < base["interactions"]
    assert runs[0.1]["far_nodes"] < runs[0.1]["far_interactions"]
    a0 = base["acc4"].reshape(-1, 4)[:, :3].astype(np.float64)
    a1 = runs[0.1]["acc4"].reshape(-1, 4)[:, :3].astype(np.float64)
    rel = np.linalg.norm(a1 - a0, axis=1) / np.linalg.norm(a0, axis=1)
    assert np.median(rel) < 1e-4 and rel.max() < 1e-2
    assert errs[0.1] < 1.05 * errs[0.0] and errs[0.2] < 1.2 * errs[0.0]


def test_far_ratio_one_particle_groups_and_systems(oracle, native):
    # Groups of one particle walked alone (box of zero size: leaves of one
    # particle at 20 bits per axis, so no leaf is cut into chunks that share
    # a walk): every accepted node is far, in every system of a batch.
    from astro_gb300 import ic

    sizes = [1, 2, 300, 1000]
    parts = [ic.plummer(s, seed=1004, system=k) for k, s in enumerate(sizes)]
    pm = np.concatenate([a for a, _ in parts])
    vr = np.concatenate([b for _, b in parts])
    near = oracle.phys_run(phys_params(group_size=1, lbits=20), pm.copy(), vr.copy(), sizes=sizes,
                           dt=0.0)
    far = oracle.phys_run(phys_params(group_size=1, lbits=20, far_ratio=0.5), pm.copy(), vr.copy(),
                          sizes=sizes, dt=0.0)
    assert far["interactions"] == near["interactions"]
    assert far["far_nodes"] == far["far_interactions"] > 0
    a0 = near["acc4"].reshape(-1, 4)[:, :3].astype(np.float64)
    a1 = far["acc4"].reshape(-1, 4)[:, :3].astype(np.float64)
    # rho = 0 for a single particle: the expansion is the node's field itself.
    rel = np.linalg.norm(a1 - a0, axis=1) / np.maximum(np.linalg.norm(a0, axis=1), 1e-30)
    assert rel.max() < 1e-5


def test_emitted_colour_known_answers(oracle):
    """emittedColor / emittedColorCenter (Octree.metal:75-106,147-187): a leaf
    sums its stars' colours and averages their positions (dividing by
    max(stars, 1e-9), so a starless leaf has centre 0); an internal node sums
    the colours of the children whose emitted alpha is above 0 and averages
    those children's centres."""
    # Two stars in one leaf cell (quantised x 1,000,000 and 1,000,100), one
    # planet in another, and a third star in the other half of the cube.
    pm, vr = particles([(0.0, 0.0, 0.0), (100.0, 0.0, 0.0), (500000.0, 0.0, 0.0),
                        (-600000.0, 0.0, 0.0)])
    ct = np.zeros(4, L.COLOR_TYPE)
    ct["color"] = [(1.0, 0.5, 0.25, 1.0), (0.5, 0.5, 0.5, 1.0), (0.9, 0.9, 0.9, 1.0),
                   (0.25, 0.25, 0.25, 0.5)]
    ct["type"] = [0, 0, 1, 0]
    out = oracle.ref_run(ref_params(), pm, vr, ct, n_tree=4, dt=0.0, steps=1, split_passes=64)
    nodes = out["nodes"]
    leaves = nodes[:out["layer_counts"][0]]
    by_mass = {int(round(float(l["totalMass"]))): l for l in leaves}
    pair = [l for l in leaves if l["totalMass"] == 2.0][0]
    assert np.array_equal(pair["emittedColor"], np.float32([1.5, 1.0, 0.75, 2.0]))
    assert np.array_equal(pair["emittedColorCenter"], np.float32([50.0, 0.0, 0.0]))
    # The planet's leaf sorts last and, by the last-leaf range of
    # aggregateLeafNodes (Octree.metal:71), sums nothing: no mass, no light.
    planet = leaves[-1]
    assert planet["totalMass"] == 0.0
    assert not planet["emittedColor"].any() and not planet["emittedColorCenter"].any()
    lone = [l for l in leaves if l["centerOfMass"][0] == -600000.0][0]
    assert np.array_equal(lone["emittedColor"], np.float32([0.25, 0.25, 0.25, 0.5]))
    assert np.array_equal(lone["emittedColorCenter"], np.float32([-600000.0, 0.0, 0.0]))
    assert len(by_mass) == 3
    root = nodes[out["layer_offsets"][-1]]
    assert np.array_equal(root["emittedColor"], np.float32([1.75, 1.25, 1.0, 2.5]))
    # Where the stars' branches meet, two children emit and their centres
    # (50 and -600000) are averaged; above it one child carries that on.
    def emitting(node):
        return [c for c in node["children"] if c != L.INVALID_CHILD
                and nodes[c]["emittedColor"][3] > 0]

    joins = [nd for nd in nodes[out["layer_counts"][0]:] if len(emitting(nd)) == 2]
    assert len(joins) == 1
    assert np.array_equal(joins[0]["emittedColorCenter"], np.float32([-299975.0, 0.0, 0.0]))
    assert np.array_equal(root["emittedColorCenter"], np.float32([-299975.0, 0.0, 0.0]))
