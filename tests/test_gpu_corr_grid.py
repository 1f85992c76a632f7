"""One MIXED cloth above the explicit-inverse limit on a cooperative grid of CTAs (the correction
kernel's cluster code with grid barriers, plan team_ctas > 16): against the oracle with the residual
gate, the displacement gate and Chebyshev-weighted iterates, and among the autotuner's candidates.
"""
import copy

import numpy as np
import pytest

from pd_gb300 import workloads as W
from tests.helpers import max_rel, oracle_twin

pytestmark = pytest.mark.gpu


def big_cfg(**kw):
    c = W._base(grid_nx=70, grid_ny=64, grid_spacing=1 / 69, max_iterations=12, shear_stiffness=900.0,
                bend_stiffness=40.0)
    c = copy.copy(c)
    c.precision = 4
    for k, v in kw.items():
        setattr(c, k, v)
    return c


@pytest.mark.parametrize("gate", ["residual", "displacement", "chebyshev"])
def test_grid_team_matches_oracle(pdg, gate):
    kw = {"residual": {}, "displacement": {"residual_tolerance": 0.0, "rel_tolerance": 1e-3},
          "chebyshev": {"cheb_mode": pdg.PD_CHEB_RHO, "cheb_start": 4, "residual_tolerance": 1e-6}}[gate]
    cfg = big_cfg(**kw)
    scene = pdg.make_grid(cfg)
    sim = pdg.Simulator(scene, cfg)
    sim.set_plan({"team_ctas": 152})
    info = sim.info()
    assert info["solve_kind"] == pdg.PD_SOLVE_SUPERNODAL32_CORRECTION and info["cluster_ctas"] == 152
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    sim.step(30)
    its_o, _ = orc.step(30)
    assert max_rel(sim.state()[0], orc.state()[0]) <= 1e-5
    its_g, _ = sim.iteration_log()
    assert np.mean(its_g == its_o) >= 0.9


def test_grid_team_repeated_launches_and_largest_team(pdg):
    """Many launches of one substep each (the barrier state carries over between launches), on
    the largest team the device holds."""
    cfg = big_cfg()
    scene = pdg.make_grid(cfg)
    sim = pdg.Simulator(scene, cfg)
    sim.set_plan({"team_ctas": 1024})  # capped at the device's cooperative capacity
    ctas = sim.info()["cluster_ctas"]
    assert ctas > 16
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    for _ in range(12):
        sim.step(1)
    orc.step(12)
    assert max_rel(sim.state()[0], orc.state()[0]) <= 1e-5


def test_autotuner_tries_grid_teams(pdg):
    cfg = big_cfg(max_iterations=6)
    sim = pdg.Simulator(pdg.make_grid(cfg), cfg)
    rep = sim.autotune(2)
    assert any(t["team_ctas"] > 16 for t in rep["tried"])
    assert rep["ms"][rep["chosen"]] == min(rep["ms"])


@pytest.mark.parametrize("p", [1, 2])
def test_fp64_supernodal_grid_team_matches_oracle(pdg, p):
    """The FP64 supernodal kernel (FP64 and FP32-projection modes) on a grid team."""
    cfg = copy.copy(W._base(grid_nx=60, grid_ny=60, grid_spacing=1 / 59, max_iterations=12, shear_stiffness=1000.0,
                            bend_stiffness=50.0))
    cfg.precision = p
    scene = pdg.make_grid(cfg)
    sim = pdg.Simulator(scene, cfg)
    sim.set_plan({"team_ctas": 152})
    assert sim.info()["cluster_ctas"] == 152 and sim.info()["solve_kind"] == pdg.PD_SOLVE_SUPERNODAL
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    sim.step(25)
    its_o, _ = orc.step(25)
    assert max_rel(sim.state()[0], orc.state()[0]) <= (1e-10 if p == 1 else 1e-5)
    assert np.array_equal(sim.iteration_log()[0], its_o) or p == 2


def test_grid_team_is_capped_by_its_slot_workspace(pdg):
    """A grid team keeps two slots per CTA in a 3n-double workspace: an 8×6 cloth (48 vertices)
    takes at most 72 CTAs, a 3×3 cloth keeps a cluster; both step like the oracle."""
    for (nx, ny), cap in (((8, 6), 72), ((3, 3), 16)):
        cfg = copy.copy(W._base(grid_nx=nx, grid_ny=ny, grid_spacing=0.05, max_iterations=4))
        cfg.precision = 1
        cfg.dense_max_vertices = -1  # the supernodal kernel (small FP64 cloths otherwise take the team kernel)
        scene = pdg.make_grid(cfg)
        sim = pdg.Simulator(scene, cfg)
        sim.set_plan({"team_ctas": 300})
        assert sim.info()["cluster_ctas"] <= cap
        orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
        sim.step(3)
        orc.step(3)
        assert max_rel(sim.state()[0], orc.state()[0]) <= 1e-10


@pytest.mark.parametrize("gate", ["residual", "displacement"])
def test_fp32_solve_grid_team_matches_oracle(pdg, gate):
    """FP32 solve + one FP64 refinement step of one cloth above the explicit-inverse limit on a grid
    team (the planner's choice for a large cloth), against the oracle."""
    kw = {"residual": {}, "displacement": {"residual_tolerance": 0.0, "rel_tolerance": 1e-3}}[gate]
    cfg = copy.copy(W._base(grid_nx=96, grid_ny=90, grid_spacing=1 / 95, max_iterations=12, shear_stiffness=900.0,
                            bend_stiffness=40.0, **kw))
    cfg.precision = 3
    scene = pdg.make_grid(cfg)
    sim = pdg.Simulator(scene, cfg)
    info = sim.info()
    assert info["solve_kind"] == pdg.PD_SOLVE_SUPERNODAL32 and info["cluster_ctas"] > 16
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    for _ in range(3):  # repeated launches: the grid barrier state carries over
        sim.step(8)
    its_o, _ = orc.step(24)
    assert max_rel(sim.state()[0], orc.state()[0]) <= 1e-5
    assert np.mean(sim.iteration_log()[0] == its_o[-8:]) >= 0.9
