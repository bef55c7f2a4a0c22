"""State files: a context saved between steps and loaded again continues
exactly as the uninterrupted context does (bit for bit), in every preset and
form; the file parses on the host and its header carries the counters."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ag(native):
    return native


def _setup(ag, case):
    from astro_gb300 import ic

    L = ag.layouts
    if case == "reference":
        p = ag.default_params(L.PRESET_REFERENCE)
        pm, vr, ct = ic.reference_scene(5, 200, 3000, seed=7)
        return p, dict(pm=pm, vr=vr, ct=ct, n_tree=205), None, 1.0 / 60
    if case == "batched":
        p = ag.default_params(L.PRESET_PHYSICAL, softening=0.01)
        sizes = [1000, 37, 4096, 1]
        parts = [ic.plummer(s, seed=3, system=k) for k, s in enumerate(sizes)]
        pm = np.concatenate([a for a, _ in parts])
        vr = np.concatenate([b for _, b in parts])
        return p, dict(pm=pm, vr=vr), sizes, 1e-3
    form = L.FORM_PRECISION if case == "precision" else L.FORM_PLAIN
    p = ag.default_params(L.PRESET_PHYSICAL, form=form, softening=0.005, lbits=12)
    pm, vr = ic.disk_bulge(20000, seed=1002)
    return p, dict(pm=pm, vr=vr), None, 5e-4


def _open(ag, p, d, sizes):
    sim = ag.Simulation(p, max_n=len(d["pm"]), max_systems=len(sizes) if sizes else 1)
    if sizes:
        sim.upload_systems(d["pm"], d["vr"], sizes)
    else:
        sim.upload(d["pm"], d["vr"], d.get("ct"), n_tree=d.get("n_tree"))
    return sim


@pytest.mark.parametrize("case", ["plain", "precision", "batched", "reference"])
def test_saved_state_resumes_bit_exactly(ag, tmp_path, case):
    L = ag.layouts
    p, d, sizes, dt = _setup(ag, case)
    path = tmp_path / f"{case}.state"
    with _open(ag, p, d, sizes) as sim:
        sim.draw(dt, 3)
        sim.save_state(path, step=3, time=3 * dt)
        sim.draw(dt, 4)
        want_pm, want_vr = sim.download()
        want_acc = sim.read_accel()
    loaded, step, t = ag.Simulation.load_state(path)
    with loaded:
        assert (step, t) == (3, pytest.approx(3 * dt))
        assert loaded.n == len(d["pm"])
        loaded.draw(dt, 4)
        got_pm, got_vr = loaded.download()
        assert np.array_equal(got_pm, want_pm)
        assert np.array_equal(got_vr, want_vr)
        assert np.array_equal(loaded.read_accel(), want_acc)
    hdr, fsizes, pm, vr, ids, types, pos64 = L.read_state(path)
    assert hdr.n == len(d["pm"]) and hdr.step == 3
    assert sorted(ids.tolist()) == list(range(hdr.n))
    assert (types is not None) == (case == "reference")
    assert (pos64 is not None) == (case == "precision")
    if sizes:
        assert fsizes.tolist() == sizes


def test_save_state_refuses_mid_step(ag, tmp_path):
    from astro_gb300 import ic

    L = ag.layouts
    p = ag.default_params(L.PRESET_PHYSICAL)
    pm, vr = ic.plummer(4096, seed=1)
    with ag.Simulation(p, max_n=4096) as sim:
        sim.upload(pm, vr)
        sim.generate_morton_codes()
        sim.sort()  # the state now sits in the sorted buffers until the traversal
        with pytest.raises(ag.AstroError):
            sim.save_state(tmp_path / "mid.state")
        sim.build_tree()
        sim.barnes_hut()
        sim.update_spheres(0.0)
        sim.save_state(tmp_path / "ok.state")


@pytest.mark.parametrize("scene", ["disk_bulge", "reference"])
def test_driver_resume_gives_identical_state_files(ag, tmp_path, scene):
    from astro_gb300 import driver

    common = ["--scene", scene, "--n", "6000", "--seed", "5", "--dt", "1e-3", "--lbits", "10"]
    a = driver.run(driver.parse(common + ["--steps", "4", "--save-every", "2",
                                          "--out", str(tmp_path / "a")]), log=lambda s: None)
    assert [r["step"] for r in a] == [2, 4]
    b = driver.run(driver.parse(["--resume", a[0]["state"], "--steps", "2", "--dt", "1e-3",
                                 "--out", str(tmp_path / "b")]), log=lambda s: None)
    assert b[-1]["step"] == 4
    assert (tmp_path / "a" / "step_000004.state").read_bytes() == \
        (tmp_path / "b" / "step_000004.state").read_bytes()


def test_reupload_in_the_same_layout_reuses_the_step(ag):
    """Uploading new particles in the layout of the last upload keeps the
    captured step; the result equals a fresh context's, and a different layout
    still rebuilds everything."""
    from astro_gb300 import ic

    L = ag.layouts
    p = ag.default_params(L.PRESET_PHYSICAL, softening=0.005, lbits=12)
    a_pm, a_vr = ic.disk_bulge(20000, seed=1)
    b_pm, b_vr = ic.plummer(20000, seed=2)
    c_pm, c_vr = ic.plummer(12345, seed=3)
    with ag.Simulation(p, max_n=20000) as sim:
        sim.upload(a_pm, a_vr)
        sim.draw(1e-3, 2)
        sim.upload(b_pm, b_vr)          # same layout
        sim.draw(1e-3, 3)
        got_b = sim.download()
        sim.upload(c_pm, c_vr)          # smaller: a new layout
        sim.draw(1e-3, 3)
        got_c = sim.download()
    for (pm, vr), got in [((b_pm, b_vr), got_b), ((c_pm, c_vr), got_c)]:
        with ag.Simulation(p, max_n=20000) as fresh:
            fresh.upload(pm, vr)
            fresh.draw(1e-3, 3)
            want = fresh.download()
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])


@pytest.mark.parametrize("case", ["plain", "batched", "reference"])
def test_oracle_started_from_a_state_file_equals_the_gpu_continuation(ag, oracle, tmp_path, case):
    """The file carries the whole state: the CPU restatement started from the
    particles read out of a saved file (in their saved slot order) steps to
    what the GPU context loaded from that file steps to, bit for bit
    (IEEE-exact traversal), so a field that saving and loading both got
    wrong would show. The precision form is left out: its FP64 master
    positions are state the restatement does not take as input."""
    L = ag.layouts
    p, d, sizes, dt = _setup(ag, case)
    if p.preset == L.PRESET_PHYSICAL:
        p = p.replace(flags=p.flags | L.FLAG_IEEE_EXACT)
    path = tmp_path / "state.bin"
    sim = _open(ag, p, d, sizes)
    sim.draw(dt, 3)
    sim.save_state(path, step=3, time=3 * dt)
    sim.close()
    hdr, ss, pm_s, vr_s, ids, types, pos64 = L.read_state(path)
    assert pos64 is None and hdr.n == len(d["pm"])

    sim2, step, _ = ag.Simulation.load_state(path)
    with sim2:
        assert step == 3
        sim2.draw(dt, 2)
        pm_g, vr_g = sim2.download()
        acc_g = sim2.read_accel()

    if p.preset == L.PRESET_REFERENCE:
        ct = np.zeros(hdr.n, L.COLOR_TYPE)
        ct["type"] = types
        ref = oracle.ref_run(p, pm_s, vr_s, ct, n_tree=hdr.n_tree, dt=dt, steps=2,
                             split_passes=64)
    else:
        ref = oracle.phys_run(p, pm_s, vr_s, sizes=[int(s) for s in ss] if hdr.nsys > 1 else None,
                              dt=dt, steps=2)
    # GPU results come back in upload order; the file's slots map to it by ids.
    assert np.array_equal(pm_g[ids], pm_s)
    assert np.array_equal(vr_g[ids], vr_s)
    assert np.array_equal(acc_g[ids], ref["acc4"])
