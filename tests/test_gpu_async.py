"""Pipelined transfers: astro_upload_async / astro_download_async.

A stream of independent inputs stepped with asynchronous uploads and
downloads must give, for every input, exactly what the synchronous calls
give (upload, step, download). A group walk that outgrows its buffers while
asynchronous transfers are queued cannot be rerun: the next synchronize
reports the overflow with the buffers grown, and the same batch then runs
through and matches."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(ag, k, n=20000):
    from astro_gb300 import ic

    out = []
    for i in range(k):
        pm, vr = ic.disk_bulge(n, seed=2000 + i)
        out.append((pm, vr))
    return out


def _params(ag, form=0):
    L = ag.layouts
    return ag.default_params(L.PRESET_PHYSICAL, form=form, softening=0.005, lbits=10,
                             far_ratio=0.2)


def _sync_results(ag, p, inputs, dt, steps):
    res = []
    with ag.Simulation(p, max_n=len(inputs[0][0])) as sim:
        for pm, vr in inputs:
            sim.upload(pm.copy(), vr.copy())
            sim.draw(dt, steps)
            res.append(sim.download())
    return res


def _pipelined(ag, p, inputs, dt, steps, shrink=False):
    L = ag.layouts
    n = len(inputs[0][0])
    outs = [(np.zeros(n, L.POSITION_MASS), np.zeros(n, L.VELOCITY_RADIUS)) for _ in inputs]
    with ag.Simulation(p, max_n=n) as sim:
        sim.upload(inputs[0][0].copy(), inputs[0][1].copy())  # the layout
        if shrink:
            from astro_gb300._native import lib

            assert lib().astro_test_walk_capacity(sim._h, 1, 2) == 0
        err = None
        for _ in range(16):  # a reported overflow: the batch again, with grown buffers
            for (pm, vr), (opm, ovr) in zip(inputs, outs):
                sim.upload_async(pm, vr)
                sim.draw(dt, steps)
                sim.download_async(opm, ovr)
            try:
                sim.synchronize()
                break
            except ag.AstroError as e:
                err = e
        else:
            raise AssertionError("the batch kept overflowing")
    return outs, err


@pytest.mark.parametrize("form,steps", [(0, 1), (1, 2)])
def test_pipelined_transfers_match_the_synchronous_calls(native, form, steps):
    ag = native
    p = _params(ag, form)
    inputs = _inputs(ag, 3)
    want = _sync_results(ag, p, inputs, 5e-4, steps)
    got, err = _pipelined(ag, p, inputs, 5e-4, steps)
    assert err is None
    for (gp, gv), (wp, wv) in zip(got, want):
        assert np.array_equal(gp, wp) and np.array_equal(gv, wv)


def test_pipelined_transfers_batched_systems(native):
    """Systems laid out by astro_upload_systems: the asynchronous uploads keep
    that layout."""
    from astro_gb300 import ic

    ag = native
    L = ag.layouts
    p = ag.default_params(L.PRESET_PHYSICAL, softening=0.01, far_ratio=0.25)
    sizes = [3000, 17, 5000, 1, 900]
    inputs = []
    for seed in (5, 6):
        parts = [ic.plummer(s, seed=seed, system=k) for k, s in enumerate(sizes)]
        inputs.append((np.concatenate([a for a, _ in parts]), np.concatenate([b for _, b in parts])))
    n = sum(sizes)
    want = []
    with ag.Simulation(p, max_n=n, max_systems=len(sizes)) as sim:
        for pm, vr in inputs:
            sim.upload_systems(pm.copy(), vr.copy(), sizes)
            sim.draw(1e-3, 1)
            want.append(sim.download())
    outs = [(np.zeros(n, L.POSITION_MASS), np.zeros(n, L.VELOCITY_RADIUS)) for _ in inputs]
    with ag.Simulation(p, max_n=n, max_systems=len(sizes)) as sim:
        sim.upload_systems(inputs[0][0].copy(), inputs[0][1].copy(), sizes)
        for (pm, vr), (opm, ovr) in zip(inputs, outs):
            sim.upload_async(pm, vr)
            sim.draw(1e-3, 1)
            sim.download_async(opm, ovr)
        sim.synchronize()
    for (gp, gv), (wp, wv) in zip(outs, want):
        assert np.array_equal(gp, wp) and np.array_equal(gv, wv)


def test_pipelined_transfers_keep_reference_types(native):
    """REFERENCE preset: the asynchronous uploads keep the particle types and
    colours of the last synchronous upload (stars, planets, dust)."""
    from astro_gb300 import ic

    ag = native
    L = ag.layouts
    p = ag.default_params(L.PRESET_REFERENCE)
    pm0, vr0, ct = ic.reference_scene(5, 200, 3000, seed=7)
    pm1, vr1, _ = ic.reference_scene(5, 200, 3000, seed=8)
    inputs = [(pm0, vr0), (pm1, vr1)]
    n = len(pm0)
    want = []
    with ag.Simulation(p, max_n=n) as sim:
        for pm, vr in inputs:
            sim.upload(pm.copy(), vr.copy(), ct, n_tree=205)
            sim.draw(1 / 60, 1)
            want.append(sim.download())
    outs = [(np.zeros(n, L.POSITION_MASS), np.zeros(n, L.VELOCITY_RADIUS)) for _ in inputs]
    with ag.Simulation(p, max_n=n) as sim:
        sim.upload(pm0.copy(), vr0.copy(), ct, n_tree=205)
        for (pm, vr), (opm, ovr) in zip(inputs, outs):
            sim.upload_async(pm, vr)
            sim.draw(1 / 60, 1)
            sim.download_async(opm, ovr)
        sim.synchronize()
    for (gp, gv), (wp, wv) in zip(outs, want):
        assert np.array_equal(gp, wp) and np.array_equal(gv, wv)


def test_overflow_under_pipelined_transfers_is_reported_then_the_batch_runs(native):
    ag = native
    p = _params(ag)
    inputs = _inputs(ag, 2)
    want = _sync_results(ag, p, inputs, 5e-4, 1)
    got, err = _pipelined(ag, p, inputs, 5e-4, 1, shrink=True)
    assert err is not None and err.status == -8  # ASTRO_ERR_DEVICE_OVERFLOW
    for (gp, gv), (wp, wv) in zip(got, want):
        assert np.array_equal(gp, wp) and np.array_equal(gv, wv)


def test_async_transfer_arguments(native):
    ag = native
    L = ag.layouts
    from astro_gb300._native import lib

    pm = np.zeros(100, L.POSITION_MASS)
    vr = np.zeros(100, L.VELOCITY_RADIUS)
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    with ag.Simulation(_params(ag), max_n=200) as sim:
        assert lib().astro_upload_async(sim._h, ptr(pm), ptr(vr), 100) == -5  # no upload yet
        sim.upload(pm, vr)
        assert lib().astro_upload_async(sim._h, ptr(pm), ptr(vr), 99) == -1   # another n
        assert lib().astro_upload_async(sim._h, None, ptr(vr), 100) == -1
        assert lib().astro_download_async(sim._h, None, None, 100) == -1
        assert lib().astro_download_async(sim._h, ptr(pm), ptr(vr), 100) == 0
        sim.synchronize()
