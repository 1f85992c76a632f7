"""Host-state stepping (pd_sim_bind_host / pd_sim_step_host): the reference's stepOnce on
mesh.positions / velocities in host memory, for a whole batch per call. Every case compares the
state after each call, bit for bit, with the same substeps driven through pd_sim_set_state →
pd_sim_step → pd_sim_get_state, for the kernels whose launches the CUDA graph captures: the MIXED
team kernel (cooperative launch), a MIXED batch whose large cloth runs as a cluster on the second
stream (fork/join inside the graph), and the reference-order FP64 kernel with the residual trace.
"""
import copy

import numpy as np
import pytest

from pd_gb300 import workloads as W
from tests.helpers import bits

pytestmark = pytest.mark.gpu


def cfg_with(cfg, precision):
    c = copy.copy(cfg)
    c.precision = precision
    return c


def vel0(s):
    return np.zeros((s.n, 3)) if s.velocities is None else np.array(s.velocities, np.float64)


def pinned_state(scenes):
    """Page-locked (n, 3) float64 arrays holding each scene's initial positions / velocities."""
    import torch
    xs, vs = [], []
    for s in scenes:
        x = torch.empty((s.n, 3), dtype=torch.float64).pin_memory().numpy()
        v = torch.empty((s.n, 3), dtype=torch.float64).pin_memory().numpy()
        x[:] = s.positions
        v[:] = vel0(s)
        xs.append(x)
        vs.append(v)
    return xs, vs


def device_path(pdg, scenes, cfgs, calls, per_call, change=None):
    """The same calls through set_state / step / state; returns the states after every call."""
    sim = pdg.Simulator(scenes, cfgs)
    xs = [np.array(s.positions, np.float64) for s in scenes]
    vs = [vel0(s) for s in scenes]
    out = []
    for c in range(calls):
        if change is not None and c == change[0]:
            change[1](sim)
        for i in range(len(scenes)):
            sim.set_state(i, xs[i], vs[i])
        sim.step(per_call[c] if isinstance(per_call, list) else per_call)
        for i in range(len(scenes)):
            xs[i], vs[i] = sim.state(i)
        out.append([(x.copy(), v.copy()) for x, v in zip(xs, vs)])
    return sim, out


def host_path(pdg, scenes, cfgs, calls, per_call, arrays, change=None):
    sim = pdg.Simulator(scenes, cfgs)
    xs, vs = arrays
    sim.bind_host(xs, vs)
    out = []
    for c in range(calls):
        if change is not None and c == change[0]:
            change[1](sim)
        sim.step_host(per_call[c] if isinstance(per_call, list) else per_call)
        out.append([(x.copy(), v.copy()) for x, v in zip(xs, vs)])
    return sim, out


def assert_same(a, b):
    for call_a, call_b in zip(a, b):
        for (xa, va), (xb, vb) in zip(call_a, call_b):
            assert np.array_equal(bits(xa), bits(xb)) and np.array_equal(bits(va), bits(vb))


def test_team_kernel_in_a_graph(pdg):
    cfg = cfg_with(W._base(grid_nx=20, grid_ny=18, grid_spacing=1 / 19, max_iterations=12,
                           shear_stiffness=1000.0, bend_stiffness=50.0), pdg.PD_PRECISION_MIXED)
    scenes = [pdg.make_grid(cfg)]
    _, ref = device_path(pdg, scenes, [cfg], 5, 1)
    sim, got = host_path(pdg, scenes, [cfg], 5, 1, pinned_state(scenes))
    info = sim.info()
    assert info["solve_kind"] == pdg.PD_SOLVE_DENSE32_TEAM
    assert info["host_state"] == pdg.PD_HOST_STATE_GRAPH
    assert_same(ref, got)


def test_batch_with_a_clustered_cloth_on_the_second_stream(pdg):
    big = cfg_with(W._base(grid_nx=92, grid_ny=92, grid_spacing=1 / 91, max_iterations=6,
                           shear_stiffness=900.0), pdg.PD_PRECISION_MIXED)
    small = cfg_with(W._base(grid_nx=17, grid_ny=23, grid_spacing=1 / 22, max_iterations=6,
                             stiffness=5000.0, bend_stiffness=100.0, pin_mode=2), pdg.PD_PRECISION_MIXED)
    tiny = cfg_with(W._base(grid_nx=16, grid_ny=16, grid_spacing=1 / 15, max_iterations=6, pin_mode=3),
                    pdg.PD_PRECISION_MIXED)
    cfgs = [small, big, tiny]
    scenes = [pdg.make_grid(c) for c in cfgs]
    _, ref = device_path(pdg, scenes, cfgs, 2, 2)
    sim, got = host_path(pdg, scenes, cfgs, 2, 2, pinned_state(scenes))
    assert sim.info(1)["solve_kind"] == pdg.PD_SOLVE_SUPERNODAL32_CORRECTION
    assert sim.info(1)["cluster_ctas"] > 1 and sim.info(0)["cluster_ctas"] == 1
    assert sim.info(0)["host_state"] == pdg.PD_HOST_STATE_GRAPH
    assert_same(ref, got)


def test_reference_order_with_trace_and_changing_substep_counts(pdg):
    cfg = cfg_with(W._base(grid_nx=10, grid_ny=8, grid_spacing=0.05, max_iterations=6, residual_tolerance=1e-6,
                           shear_stiffness=700.0), pdg.PD_PRECISION_FP64_EXACT)
    scenes = [pdg.make_grid(cfg)]
    counts = [3, 1, 3]
    ref_sim = pdg.Simulator(scenes, [cfg])
    ref_sim.set_residual_trace(True)
    x, v = np.array(scenes[0].positions), vel0(scenes[0])
    ref = []
    for k in counts:
        ref_sim.set_state(0, x, v)
        ref_sim.step(k)
        x, v = ref_sim.state(0)
        ref.append([(x.copy(), v.copy())])
    sim = pdg.Simulator(scenes, [cfg])
    sim.set_residual_trace(True)
    arrays = pinned_state(scenes)
    sim.bind_host(*arrays)
    got = []
    for k in counts:
        sim.step_host(k)
        got.append([(arrays[0][0].copy(), arrays[1][0].copy())])
    assert_same(ref, got)
    assert np.array_equal(bits(sim.residual_trace(0)), bits(ref_sim.residual_trace(0)))
    assert np.array_equal(sim.iteration_log(0)[0], ref_sim.iteration_log(0)[0])


def test_refactorization_between_calls(pdg):
    """A stiffness change re-uploads the arena: the next call must capture a new graph."""
    cfg = cfg_with(W._base(grid_nx=12, grid_ny=12, grid_spacing=1 / 11, max_iterations=8), pdg.PD_PRECISION_MIXED)
    scenes = [pdg.make_grid(cfg)]
    k = np.asarray(scenes[0].edge_stiffness) * 1.7
    change = (2, lambda sim: sim.set_edge_stiffness(k, 0))
    _, ref = device_path(pdg, scenes, [cfg], 4, 1, change)
    _, got = host_path(pdg, scenes, [cfg], 4, 1, pinned_state(scenes), change)
    assert_same(ref, got)


def test_pageable_arrays_copy_per_array(pdg):
    cfg = cfg_with(W._base(grid_nx=9, grid_ny=11, grid_spacing=0.05, max_iterations=5), pdg.PD_PRECISION_FP64)
    scenes = [pdg.make_grid(cfg), pdg.make_grid(cfg)]
    _, ref = device_path(pdg, scenes, [cfg, cfg], 3, 2)
    arrays = ([np.array(s.positions, np.float64) for s in scenes], [vel0(s) for s in scenes])
    sim, got = host_path(pdg, scenes, [cfg, cfg], 3, 2, arrays)
    assert sim.info()["host_state"] == pdg.PD_HOST_STATE_COPIES
    assert_same(ref, got)


def test_zero_substeps_round_trip_and_errors(pdg):
    cfg = cfg_with(W._base(grid_nx=6, grid_ny=5, grid_spacing=0.05, max_iterations=3), pdg.PD_PRECISION_FP64_EXACT)
    scene = pdg.make_grid(cfg)
    sim = pdg.Simulator(scene, cfg)
    with pytest.raises(pdg.PdError):
        sim.step_host(1)  # nothing bound
    xs, vs = pinned_state([scene])
    sim.bind_host(xs, vs)
    before = xs[0].copy()
    sim.step_host(0)
    assert np.array_equal(bits(xs[0]), bits(before))
    xs[0][3, 1] = np.nan
    with pytest.raises(pdg.PdError) as e:
        sim.step_host(1)
    assert e.value.code == 1  # PD_ERR_INVALID_ARGUMENT
    sim.bind_host(None, None)
    assert sim.info()["host_state"] == pdg.PD_HOST_STATE_NONE
    with pytest.raises(ValueError):
        sim.bind_host([np.zeros((3, 3))], [np.zeros((3, 3))])
