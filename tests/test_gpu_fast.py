"""FP64 supernodal mode (PD_PRECISION_FP64) against the CPU oracle.

Its solve sums in a different order than the reference (tree-level reductions, FMA), so it is
held to a tolerance: positions within 1e-10 relative of the oracle (max |Δx| / max |x|) after the
full 600-substep scene, with identical per-substep iteration counts (the gate decides the same).
"""
import copy

import numpy as np
import pytest

from pd_gb300 import workloads as W
from tests.helpers import max_rel, oracle_twin

pytestmark = pytest.mark.gpu

TOL_POS = 1e-10


def fast(cfg, ctas=0):
    c = copy.copy(cfg)
    c.precision = 1
    c.cluster_ctas = ctas
    return c


def test_solve_matches_oracle(pdg):
    scenes, cfg, _ = W.cloth40_full()
    sim = pdg.Simulator(scenes[0], fast(cfg))
    orc = oracle_twin(scenes[0], cfg, perm=sim.factor()["perm"])
    rng = np.random.default_rng(5)
    for _ in range(3):
        b = rng.standard_normal((scenes[0].n, 3))
        assert max_rel(sim.solve(b), orc.solve(b)) < 1e-13


@pytest.mark.parametrize("ctas", [1, 4, 16])
@pytest.mark.parametrize("name,substeps", [("cloth40_plain", 600), ("cloth40_full", 120)])
def test_trajectory_within_tolerance(pdg, name, substeps, ctas):
    scenes, cfg, _ = W.WORKLOADS[name]()
    sim = pdg.Simulator(scenes[0], fast(cfg, ctas))
    orc = oracle_twin(scenes[0], cfg, perm=sim.factor()["perm"])
    sim.step(substeps)
    it_g, _ = sim.iteration_log()
    it_o, _ = orc.step(substeps)
    assert np.array_equal(it_g, it_o)
    xg, vg = sim.state()
    xo, vo = orc.state()
    assert max_rel(xg, xo) < TOL_POS
    assert max_rel(vg, vo) < 1e-7
    pins = np.flatnonzero(scenes[0].pinned)
    assert np.array_equal(xg[pins], scenes[0].positions[pins])


def test_cluster_without_replicas_matches_oracle(pdg):
    """A 60×60 cloth needs more than the shared-memory replicas hold: the cluster keeps its
    workspaces in L2 instead."""
    cfg = fast(W._base(grid_nx=60, grid_ny=60, grid_spacing=1 / 59, max_iterations=10, shear_stiffness=1000.0,
                       bend_stiffness=50.0), 16)
    scene = pdg.make_grid(cfg)
    sim = pdg.Simulator(scene, cfg)
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    sim.step(40)
    it_o, _ = orc.step(40)
    assert np.array_equal(sim.iteration_log()[0], it_o)
    assert max_rel(sim.state()[0], orc.state()[0]) < TOL_POS


@pytest.mark.parametrize("ctas", [1, 8])
def test_batch_fast_matches_oracle(pdg, ctas):
    scenes, cfgs, _ = W.batch(count=6, seed=21, max_side=48)
    cfgs = [fast(c, ctas) for c in cfgs]
    sim = pdg.Simulator(scenes, cfgs)
    sim.step(30)
    for i, (s, c) in enumerate(zip(scenes, cfgs)):
        orc = oracle_twin(s, c, perm=sim.factor(i)["perm"])
        orc.step(30)
        xg, _ = sim.state(i)
        xo, _ = orc.state()
        assert max_rel(xg, xo) < TOL_POS, i


@pytest.mark.parametrize("ctas", [1, 16])
def test_gate_decisions_match_in_fast_mode(pdg, ctas):
    cfg = fast(W._base(grid_nx=12, grid_ny=12, grid_spacing=0.05, max_iterations=30, residual_tolerance=0.3,
                       velocity_damping=0.02), ctas)
    scene = pdg.make_grid(cfg)
    sim = pdg.Simulator(scene, cfg)
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    sim.step(200)
    it_o, _ = orc.step(200)
    it_g, _ = sim.iteration_log()
    assert np.array_equal(it_g, it_o) and it_o.min() < 30
    assert max_rel(sim.state()[0], orc.state()[0]) < TOL_POS
