"""Group-walk buffers that are too small for the walk.

The walk keeps counting the list blocks and frontier words it needs, the
evaluation skips (no force is written, no particle moves), and the host
grows the buffers from those counts and runs the skipped steps again, or
at once the stage call's traversal. The results must equal those of a
context whose buffers were large enough from the start, bit for bit. The
small buffers are set through astro_test_walk_capacity; every write of the
walk stays inside the buffers it was given."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _capacity(sim, blocks=0, frontier=0):
    """Sets the walk's buffers (blocks, frontier words; 0 keeps one) when
    asked; returns their sizes and the steps run again so far."""
    from astro_gb300._native import lib

    if blocks or frontier:
        assert lib().astro_test_walk_capacity(sim._h, blocks, frontier) == 0
    b, f, r = ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_uint64()
    assert lib().astro_read_walk_buffers(sim._h, ctypes.byref(b), ctypes.byref(f),
                                         ctypes.byref(r)) == 0
    return b.value, f.value, r.value


def _case(ag, form, batched, no_graph, node_list=False):
    from astro_gb300 import ic

    L = ag.layouts
    flags = L.FLAG_OPEN_DELTA | L.FLAG_QUADRUPOLE | (L.FLAG_NO_GRAPH if no_graph else 0)
    p = ag.default_params(L.PRESET_PHYSICAL, form=form, softening=0.005, lbits=10, far_ratio=0.2,
                          flags=flags, walk_frontier=1 if node_list else 0)
    if batched:
        sizes = [3000, 17, 9000, 1, 5000]
        parts = [ic.plummer(s, seed=11, system=k) for k, s in enumerate(sizes)]
        return p, np.concatenate([a for a, _ in parts]), np.concatenate([b for _, b in parts]), sizes
    pm, vr = ic.disk_bulge(20000, seed=1003)
    return p, pm, vr, None


def _run(ag, p, pm, vr, sizes, steps, blocks=0, frontier=0, sync=True):
    with ag.Simulation(p, max_n=len(pm), max_systems=len(sizes) if sizes else 1) as sim:
        if sizes:
            sim.upload_systems(pm, vr, sizes)
        else:
            sim.upload(pm, vr)
        if blocks or frontier:
            _capacity(sim, blocks, frontier)
        sim.draw(5e-4, steps)
        if sync:
            sim.synchronize()
        out = dict(state=sim.download(), acc=sim.read_accel(), stats=sim.read_stats(),
                   far=sim.read_far_stats(), capacity=_capacity(sim))
    return out


def test_readbacks_wait_for_the_rerun(native):
    """A readback right after the steps (no explicit synchronize) sees the
    state of the rerun steps, not the state the skipped evaluations left."""
    ag = native
    L = ag.layouts
    p, pm, vr, sizes = _case(ag, L.FORM_PLAIN, False, False)
    want = _run(ag, p, pm.copy(), vr.copy(), sizes, 2)
    got = _run(ag, p, pm.copy(), vr.copy(), sizes, 2, 1, 2, sync=False)
    for a, b in zip(got["state"], want["state"]):
        assert np.array_equal(a, b)
    assert np.array_equal(got["acc"], want["acc"]) and got["capacity"][2] >= 2


@pytest.mark.parametrize("form,batched,no_graph,blocks,frontier,node_list", [
    ("plain", False, False, 1, 0, False),      # the list pool: one block
    ("plain", False, False, 0, 2, False),      # the frontier: one run
    ("plain", False, False, 0, 2, True),       # the node-list frontier: two nodes
    ("precision", False, True, 1, 2, False),   # both, steps launched one by one
    ("plain", True, False, 40, 8, False),      # systems batched into one step
])
def test_steps_rerun_after_the_walk_ran_out_of_room(native, form, batched, no_graph, blocks,
                                                    frontier, node_list):
    ag = native
    L = ag.layouts
    p, pm, vr, sizes = _case(ag, L.FORM_PRECISION if form == "precision" else L.FORM_PLAIN,
                             batched, no_graph, node_list)
    want = _run(ag, p, pm.copy(), vr.copy(), sizes, 3)
    got = _run(ag, p, pm.copy(), vr.copy(), sizes, 3, blocks, frontier)
    for a, b in zip(got["state"], want["state"]):
        assert np.array_equal(a, b)
    assert np.array_equal(got["acc"], want["acc"])
    assert got["stats"] == want["stats"] and got["far"] == want["far"]
    if blocks:
        assert got["capacity"][0] > blocks
    if frontier:
        assert got["capacity"][1] > frontier
    assert want["capacity"][2] == 0 and got["capacity"][2] >= 3  # every step ran again


def test_stage_traversal_reruns_at_once(native):
    """astro_traverse outside a step: the traversal runs again before the
    call returns, with the sorted state and the tree still in place."""
    ag = native
    L = ag.layouts
    p, pm, vr, _ = _case(ag, L.FORM_PLAIN, False, False)
    out = []
    for cap in (None, (1, 2)):
        with ag.Simulation(p, max_n=len(pm)) as sim:
            sim.upload(pm.copy(), vr.copy())
            if cap:
                _capacity(sim, *cap)
            sim.generate_morton_codes()
            sim.sort()
            sim.build_tree()
            sim.barnes_hut()
            out.append((sim.read_accel(), sim.read_stats(), sim.download(), _capacity(sim)))
    (acc0, st0, s0, _), (acc1, st1, s1, c1) = out
    assert np.array_equal(acc0, acc1) and st0 == st1
    for a, b in zip(s0, s1):
        assert np.array_equal(a, b)
    assert c1[0] > 1 and c1[1] > 2 and c1[2] >= 1


def test_capacity_hook_rejects_bad_sizes(native):
    ag = native
    L = ag.layouts
    from astro_gb300._native import lib

    with ag.Simulation(ag.default_params(L.PRESET_PHYSICAL), max_n=64) as sim:
        assert lib().astro_test_walk_capacity(sim._h, 0, 1) == -1  # invalid argument
        assert lib().astro_test_walk_capacity(sim._h, 0, 7) == -1  # odd: runs are 8 bytes
    with ag.Simulation(ag.default_params(L.PRESET_REFERENCE), max_n=64) as sim:
        assert lib().astro_test_walk_capacity(sim._h, 4, 0) == -5  # state
