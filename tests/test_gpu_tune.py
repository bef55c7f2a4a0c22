"""The library's native autotuner (astro_autotune_ex) and the batched step
entry (astro_step_batched), through the C ABI."""
import ctypes
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ag(native):
    return native


def _same(a, b):
    return np.isclose(float(a), float(b), rtol=1e-6, atol=0.0)


def test_autotune_applies_its_choice_within_its_bounds(ag, tmp_path):
    from astro_gb300 import autotune, ic

    L = ag.layouts
    pm, vr = ic.plummer(16384, seed=1001)
    p = ag.default_params(L.PRESET_PHYSICAL, lbits=10, softening=0.01)
    with ag.Simulation(p, max_n=len(pm)) as sim:
        sim.upload(pm, vr)
        pm0, vr0 = sim.download()
        path = tmp_path / "tune.json"
        res = sim.autotune(path=path, samples=256)
        assert json.loads(path.read_text())["knobs"] == res["knobs"]
        k = res["knobs"]
        q = sim.params
        assert (q.lbits, q.bucket, q.group_size, q.block_warps, q.sort_variant) == (
            k["lbits"], k["bucket"], k["group_size"], k["block_warps"], k["sort_variant"])
        assert _same(q.far_ratio, k["far_ratio"]) and _same(q.open_delta_weight, k["open_delta_weight"])
        # The chosen setting is within the search's error bound and no slower
        # than the start.
        start = res["trials"][0]
        assert res["median_error"] <= res["error_bound"]
        assert res["ms"] <= start["ms"]
        assert res["accuracy_knob_bound"] <= res["error_bound"]
        # Every trial moves knobs only to the documented candidate values.
        for t in res["trials"]:
            for knob in autotune.KNOBS:
                v = t["knobs"][knob]
                allowed = [start["knobs"][knob]] + list(autotune.candidates(knob, len(pm)))
                if knob == "far_ratio":
                    allowed.append(0.0)
                if knob == "open_delta_weight":
                    allowed.append(1.0)
                assert any(_same(v, a) for a in allowed), (knob, v)
        # Steps with dt = 0: the particles are unchanged; the context still steps.
        pm1, vr1 = sim.download()
        assert np.array_equal(pm0, pm1) and np.array_equal(vr0, vr1)
        sim.draw(1e-3, 2)
        sim.synchronize()


def test_autotune_refuses_the_reference_preset_and_an_empty_context(ag):
    from astro_gb300 import ic

    L = ag.layouts
    pm, vr, ct = ic.reference_scene(5, 200, 1000, seed=7)
    with ag.Simulation(ag.default_params(L.PRESET_REFERENCE), max_n=len(pm)) as sim:
        with pytest.raises(ag.AstroError):
            sim.autotune()
        sim.upload(pm, vr, ct, n_tree=205)
        with pytest.raises(ag.AstroError):
            sim.autotune()
        assert sim.params.preset == L.PRESET_REFERENCE


def test_step_batched_equals_step(ag):
    from astro_gb300 import ic

    L = ag.layouts
    sizes = [1000, 2000, 517, 1]
    parts = [ic.plummer(s, seed=9, system=k) for k, s in enumerate(sizes)]
    pm = np.concatenate([a for a, _ in parts])
    vr = np.concatenate([b for _, b in parts])
    p = ag.default_params(L.PRESET_PHYSICAL, softening=0.01, far_ratio=0.2)
    outs = []
    for batched in (False, True):
        with ag.Simulation(p, max_n=len(pm), max_systems=len(sizes)) as sim:
            sim.upload_systems(pm, vr, sizes)
            if batched:
                sim.draw_batched(1e-3, 3, sizes)
                with pytest.raises(ag.AstroError):
                    sim.draw_batched(1e-3, 1, [1000, 2000, 518])
                with pytest.raises(ag.AstroError):
                    sim.draw_batched(1e-3, 1, sizes[:3])
            else:
                sim.draw(1e-3, 3)
            outs.append(sim.download())
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_autotune_failure_keeps_the_context(ag, tmp_path):
    # An unwritable result path fails the call after the search; the
    # context keeps its parameters and particles and still steps.
    from astro_gb300 import ic

    L = ag.layouts
    pm, vr = ic.plummer(4096, seed=11)
    p = ag.default_params(L.PRESET_PHYSICAL, lbits=8, softening=0.01)
    with ag.Simulation(p, max_n=len(pm)) as sim:
        sim.upload(pm, vr)
        pm0, vr0 = sim.download()
        with pytest.raises(ag.AstroError):
            sim.autotune(path=tmp_path / "missing_dir" / "tune.json", samples=64)
        q = ag.Params()
        assert ag._native.lib().astro_get_params(sim._h, ctypes.byref(q)) == 0
        assert bytes(q) == bytes(p)
        pm1, vr1 = sim.download()
        assert np.array_equal(pm0, pm1) and np.array_equal(vr0, vr1)
        sim.draw(1e-3, 1)
        sim.synchronize()
