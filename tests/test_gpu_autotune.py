"""Launch-plan autotuner (pd_sim_autotune / pd_sim_set_plan): tuning leaves the simulation where
it was, the kept plan is the fastest candidate timed, the tuned handle still matches the oracle
within its mode's bar, and a plan handed to a fresh handle reproduces the tuned handle bit for bit.
"""
import copy

import numpy as np
import pytest

from pd_gb300 import workloads as W
from tests.helpers import bits, max_rel, oracle_twin

pytestmark = pytest.mark.gpu

TOL = {0: 0.0, 1: 1e-10, 4: 1e-5}


def cfg_with(cfg, precision):
    c = copy.copy(cfg)
    c.precision = precision
    return c


def snapshot(sim):
    return [(sim.state(i), sim.stats(i)) for i in range(sim.count)]


def assert_unchanged(before, after):
    for ((xa, va), sa), ((xb, vb), sb) in zip(before, after):
        assert np.array_equal(bits(xa), bits(xb)) and np.array_equal(bits(va), bits(vb))
        assert sa == sb or (np.isnan(sa["last_residual"]) and np.isnan(sb["last_residual"]))


def tune_and_check(pdg, scenes, cfgs, p, warm=3, tune_steps=3, steps=6, min_candidates=1):
    sim = pdg.Simulator(scenes, cfgs)
    sim.step(warm)  # tune from a moving state, not the rest pose
    before = snapshot(sim)
    rep = sim.autotune(tune_steps)
    assert len(rep["tried"]) >= min_candidates
    assert rep["ms"][rep["chosen"]] == min(rep["ms"])
    assert_unchanged(before, snapshot(sim))
    assert sim.plan() == rep["tried"][rep["chosen"]]
    # the tuned handle against the oracle from the same start
    sim.step(steps)
    for i, (s, c) in enumerate(zip(scenes, cfgs)):
        orc = oracle_twin(s, c, perm=sim.factor(i)["perm"])
        orc.step(warm + steps)
        assert max_rel(sim.state(i)[0], orc.state()[0]) <= max(TOL[p], 1e-15), i
    # the kept plan handed to a fresh handle at the same point reproduces the tuned handle
    fresh = pdg.Simulator(scenes, cfgs)
    fresh.step(warm)
    fresh.set_plan(rep["tried"][rep["chosen"]])
    fresh.step(steps)
    for i in range(len(scenes)):
        assert np.array_equal(bits(fresh.state(i)[0]), bits(sim.state(i)[0])), i
    return rep


def test_team_kernel_team_sizes(pdg):
    cfg = cfg_with(W._base(grid_nx=24, grid_ny=24, grid_spacing=1 / 23, max_iterations=10, shear_stiffness=1000.0,
                           bend_stiffness=50.0), 4)
    scene = pdg.make_grid(cfg)
    rep = tune_and_check(pdg, [scene], [cfg], 4, min_candidates=3)
    assert rep["tried"][0]["team_ctas"] > rep["tried"][1]["team_ctas"] >= 2


def test_batch_cluster_threshold_and_size(pdg):
    big = cfg_with(W._base(grid_nx=92, grid_ny=92, grid_spacing=1 / 91, max_iterations=5, shear_stiffness=900.0), 4)
    mid = cfg_with(W._base(grid_nx=70, grid_ny=64, grid_spacing=1 / 69, max_iterations=5, stiffness=5000.0,
                           bend_stiffness=100.0, pin_mode=2), 4)
    tiny = cfg_with(W._base(grid_nx=16, grid_ny=16, grid_spacing=1 / 15, max_iterations=5, pin_mode=3), 4)
    cfgs = [mid, big, tiny]
    scenes = [pdg.make_grid(c) for c in cfgs]
    rep = tune_and_check(pdg, scenes, cfgs, 4, tune_steps=2, steps=4, min_candidates=8)
    assert any(t["big_cluster_ctas"] == 8 for t in rep["tried"])
    assert any(t["latency_scale"] != 1.0 for t in rep["tried"])


def test_fp64_supernodal_cluster_sizes(pdg):
    cfg = cfg_with(W._base(grid_nx=30, grid_ny=28, grid_spacing=1 / 29, max_iterations=8, shear_stiffness=1000.0), 1)
    scene = pdg.make_grid(cfg)
    rep = tune_and_check(pdg, [scene], [cfg], 1, min_candidates=5)
    assert {t["team_ctas"] for t in rep["tried"]} >= {1, 16}


def test_reference_order_has_one_candidate(pdg):
    cfg = cfg_with(W._base(grid_nx=8, grid_ny=7, grid_spacing=0.05, max_iterations=5), 0)
    scene = pdg.make_grid(cfg)
    rep = tune_and_check(pdg, [scene], [cfg], 0)
    assert len(rep["tried"]) == 1 and rep["chosen"] == 0


def test_plan_validation(pdg):
    cfg = cfg_with(W._base(grid_nx=8, grid_ny=7, grid_spacing=0.05, max_iterations=5), 1)
    sim = pdg.Simulator(pdg.make_grid(cfg), cfg)
    for bad in ({"team_ctas": -1}, {"big_cluster_ctas": 1}, {"big_cluster_ctas": 32}, {"latency_scale": -2.0},
                {"latency_scale": float("nan")}):
        with pytest.raises(pdg.PdError):
            sim.set_plan(bad)
    sim.set_plan({"team_ctas": 2})
    assert sim.plan()["team_ctas"] == 2
    with pytest.raises(pdg.PdError):
        sim.autotune(0)
