"""Reduced-precision modes against the FP64 CPU oracle.

FP32 projection (accumulated in FP64), FP32 solve + one FP64 refinement step, and both together
must keep positions within 1e-5 relative (max |Δx| / max |x|) of the FP64 oracle after the full
600-substep scenes; the report also carries the error so it can be stated with every result.
"""
import copy

import numpy as np
import pytest

from pd_gb300 import workloads as W
from tests.helpers import max_rel, oracle_twin

pytestmark = pytest.mark.gpu

TOL_POS = 1e-5
MODES = {"fp32-projection": 2, "fp32-solve": 3, "mixed": 4}


# (CTAs per cloth, dense_max_vertices): one CTA; a cluster whose CTAs each run the supernodal
# FP32 solve; 16 CTAs splitting the rows of the explicit FP32 inverse (a cluster for FP32_SOLVE,
# a team with the correction-form solve for MIXED); every SM on the cloth (MIXED team)
STRATEGIES = {"one-cta": (1, 0), "cluster-supernodal": (16, -1), "cluster-dense": (16, 0), "auto": (0, 0)}


def with_mode(cfg, mode, ctas=0, dense=0):
    c = copy.copy(cfg)
    c.precision = MODES[mode]
    c.cluster_ctas = ctas
    c.dense_max_vertices = dense
    return c


def expected_kind(pdg, mode, ctas, dense):
    m = MODES[mode]
    if m == pdg.PD_PRECISION_FP32_PROJECTION:  # the FP64 team kernel unless a cluster is asked for
        return pdg.PD_SOLVE_DENSE64_TEAM if (ctas == 0 and dense >= 0) else pdg.PD_SOLVE_SUPERNODAL
    if m == pdg.PD_PRECISION_MIXED:  # a team on the explicit inverse, else one CTA in correction form
        return pdg.PD_SOLVE_DENSE32_TEAM if (ctas != 1 and dense >= 0) else pdg.PD_SOLVE_SUPERNODAL32_CORRECTION
    return pdg.PD_SOLVE_SUPERNODAL32 if (ctas == 1 or dense < 0) else pdg.PD_SOLVE_DENSE32


@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("strategy", list(STRATEGIES))
def test_plain_cloth_600_substeps(pdg, mode, strategy):
    scenes, cfg, substeps = W.cloth40_plain()
    ctas, dense = STRATEGIES[strategy]
    if MODES[mode] == pdg.PD_PRECISION_FP32_PROJECTION and strategy == "cluster-dense":
        pytest.skip("a 16-CTA request keeps the FP64 supernodal cluster: the same as cluster-supernodal")
    sim = pdg.Simulator(scenes[0], with_mode(cfg, mode, ctas, dense))
    assert sim.info()["solve_kind"] == expected_kind(pdg, mode, ctas, dense)
    orc = oracle_twin(scenes[0], cfg, perm=sim.factor()["perm"])
    sim.step(substeps)
    orc.step(substeps)
    err = max_rel(sim.state()[0], orc.state()[0])
    assert err < TOL_POS, err
    pins = np.flatnonzero(scenes[0].pinned)
    assert np.array_equal(sim.state()[0][pins], scenes[0].positions[pins])


@pytest.mark.parametrize("mode", ["mixed", "fp32-solve", "fp32-projection"])
@pytest.mark.parametrize("strategy", list(STRATEGIES))
def test_full_cloth_600_substeps(pdg, mode, strategy):
    scenes, cfg, substeps = W.cloth40_full()
    ctas, dense = STRATEGIES[strategy]
    if MODES[mode] == pdg.PD_PRECISION_FP32_PROJECTION and strategy == "cluster-dense":
        pytest.skip("a 16-CTA request keeps the FP64 supernodal cluster: the same as cluster-supernodal")
    sim = pdg.Simulator(scenes[0], with_mode(cfg, mode, ctas, dense))
    assert sim.info()["solve_kind"] == expected_kind(pdg, mode, ctas, dense)
    orc = oracle_twin(scenes[0], cfg, perm=sim.factor()["perm"])
    sim.step(substeps)
    it_o, _ = orc.step(substeps)
    err = max_rel(sim.state()[0], orc.state()[0])
    assert err < TOL_POS, err
    it_g, _ = sim.iteration_log()
    assert np.mean(it_g == it_o) > 0.99  # the gate rarely, if ever, decides differently


@pytest.mark.parametrize("dense", [0, -1])
def test_batch_mixed(pdg, dense):
    """Eight cloths of 16–64 vertices a side, 16-CTA clusters (dense inverse or supernodal)."""
    scenes, cfgs, _ = W.batch(count=8, seed=33, max_side=64)
    sim = pdg.Simulator(scenes, [with_mode(c, "mixed", 0, dense) for c in cfgs])
    sim.step(100)
    for i, (s, c) in enumerate(zip(scenes, cfgs)):
        orc = oracle_twin(s, c, perm=sim.factor(i)["perm"])
        orc.step(100)
        assert max_rel(sim.state(i)[0], orc.state()[0]) < TOL_POS, i


def test_large_cloth_uses_global_workspace(pdg):
    """A 90×90 cloth is above the explicit-inverse limit and its solve vectors do not fit shared
    memory: one CTA in correction form with L2 workspaces."""
    cfg = with_mode(W._base(grid_nx=90, grid_ny=90, grid_spacing=1 / 89, max_iterations=10,
                            shear_stiffness=1000.0), "mixed")
    scene = pdg.make_grid(cfg)
    sim = pdg.Simulator(scene, cfg)
    assert sim.info()["solve_kind"] == pdg.PD_SOLVE_SUPERNODAL32_CORRECTION
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    sim.step(30)
    orc.step(30)
    assert max_rel(sim.state()[0], orc.state()[0]) < TOL_POS


@pytest.mark.parametrize("strategy", ["cluster-dense", "auto"])
def test_team_pin_move(pdg, strategy):
    """Handles dragged between steps: the first iterate's matrix couples neighbours at the new q
    while the projections still see the old pin positions."""
    scenes, cfg, _ = W.cloth40_plain()
    scene = scenes[0]
    ctas, dense = STRATEGIES[strategy]
    sim = pdg.Simulator(scene, with_mode(cfg, "mixed", ctas, dense))
    assert sim.info()["solve_kind"] == pdg.PD_SOLVE_DENSE32_TEAM
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    pins = np.flatnonzero(scene.pinned)
    sim.step(20)
    orc.step(20)
    q = scene.positions.copy()
    q[pins, 0] += 0.05
    q[pins, 2] -= 0.03
    sim.set_pin_positions(q)
    orc.set_pin_positions(q)
    for _ in range(3):
        sim.step(20)
        orc.step(20)
        assert max_rel(sim.state()[0], orc.state()[0]) < TOL_POS
    x, v = sim.state()
    assert np.array_equal(x[pins], q[pins]) and not np.any(v[pins])


def test_team_gates(pdg):
    """Team kernel: residual gate that fires, displacement gate, and zero iterations."""
    cases = [
        W._base(grid_nx=12, grid_ny=12, grid_spacing=0.05, max_iterations=30, residual_tolerance=0.3,
                velocity_damping=0.02),
        W._base(grid_nx=10, grid_ny=14, grid_spacing=0.05, max_iterations=25, residual_tolerance=0.0,
                rel_tolerance=5e-2),
        W._base(grid_nx=10, grid_ny=10, grid_spacing=0.05, max_iterations=0),
    ]
    for cfg in cases:
        scene = pdg.make_grid(cfg)
        sim = pdg.Simulator(scene, with_mode(cfg, "mixed"))
        assert sim.info()["solve_kind"] == pdg.PD_SOLVE_DENSE32_TEAM
        orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
        sim.step(100)
        it_o, cv_o = orc.step(100)
        it_g, cv_g = sim.iteration_log()
        assert max_rel(sim.state()[0], orc.state()[0]) < TOL_POS
        assert np.mean(it_g == it_o) > 0.95 and np.mean(cv_g == cv_o) > 0.95
        st = sim.stats()
        if cfg.max_iterations == 0:
            assert st["iterations_used"] == 0 and not np.any(it_g)


def test_team_batch_and_repeated_launches(pdg):
    """Several cloths share the SMs; many short launches reuse the team barrier counters."""
    scenes, cfgs, _ = W.batch(count=6, seed=91, max_side=40)
    sim = pdg.Simulator(scenes, [with_mode(c, "mixed") for c in cfgs])
    assert sim.info()["solve_kind"] == pdg.PD_SOLVE_DENSE32_TEAM
    assert sim.info()["cluster_ctas"] >= 2
    for _ in range(25):
        sim.step(2)
    sim.synchronize()
    for i, (s, c) in enumerate(zip(scenes, cfgs)):
        orc = oracle_twin(s, c, perm=sim.factor(i)["perm"])
        orc.step(50)
        assert max_rel(sim.state(i)[0], orc.state()[0]) < TOL_POS, i


@pytest.mark.parametrize("strategy", ["one-cta", "cluster-supernodal"])
def test_correction_gates_and_pins(pdg, strategy):
    """One-CTA correction kernel: residual gate that fires, displacement gate, zero iterations,
    and pin drags."""
    ctas, dense = STRATEGIES[strategy]
    cases = [
        W._base(grid_nx=12, grid_ny=12, grid_spacing=0.05, max_iterations=30, residual_tolerance=0.3,
                velocity_damping=0.02),
        W._base(grid_nx=10, grid_ny=14, grid_spacing=0.05, max_iterations=25, residual_tolerance=0.0,
                rel_tolerance=5e-2),
        W._base(grid_nx=10, grid_ny=10, grid_spacing=0.05, max_iterations=0),
    ]
    for cfg in cases:
        scene = pdg.make_grid(cfg)
        sim = pdg.Simulator(scene, with_mode(cfg, "mixed", ctas, dense))
        assert sim.info()["solve_kind"] == pdg.PD_SOLVE_SUPERNODAL32_CORRECTION
        orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
        sim.step(60)
        it_o, cv_o = orc.step(60)
        if cfg.max_iterations:
            pins = np.flatnonzero(scene.pinned)
            q = scene.positions.copy()
            q[pins, 0] += 0.03
            sim.set_pin_positions(q)
            orc.set_pin_positions(q)
            sim.step(40)
            it2, cv2 = orc.step(40)
            it_o, cv_o = np.concatenate([it_o, it2]), np.concatenate([cv_o, cv2])
        assert max_rel(sim.state()[0], orc.state()[0]) < TOL_POS
        it_g, cv_g = sim.iteration_log()
        assert np.mean(it_g == it_o[-len(it_g):]) > 0.95


def test_batch_with_large_cloths_on_clusters(pdg):
    """A MIXED batch whose large cloths run as 4-CTA clusters on a second stream while the small
    ones run one CTA each: every cloth still matches the oracle."""
    sides = [(92, 92), (20, 24), (96, 90), (16, 40), (30, 30)]
    scenes, cfgs = [], []
    for nx, ny in sides:
        cfg = with_mode(W._base(grid_nx=nx, grid_ny=ny, grid_spacing=1.0 / (max(nx, ny) - 1), max_iterations=10,
                                shear_stiffness=900.0), "mixed")
        scenes.append(pdg.make_grid(cfg))
        cfgs.append(cfg)
    sim = pdg.Simulator(scenes, cfgs)
    assert sim.info(0)["solve_kind"] == pdg.PD_SOLVE_SUPERNODAL32_CORRECTION
    for _ in range(2):
        sim.step(10)
    sim.synchronize()
    for i, (s, c) in enumerate(zip(scenes, cfgs)):
        orc = oracle_twin(s, c, perm=sim.factor(i)["perm"])
        orc.step(20)
        assert max_rel(sim.state(i)[0], orc.state()[0]) < TOL_POS, i


@pytest.mark.parametrize("threads", [512, 1024])
def test_batch_as_a_work_table(pdg, threads):
    """The MIXED batch as a work table (plan work_threads 512 / 1024): resident CTAs take the cloths
    largest first from a counter, which restarts every launch. Every cloth matches the oracle after
    twelve one-substep launches, and a second handle stepped the same way gives the same bits,
    whichever CTA took which cloth."""
    sides = [(92, 92), (20, 24), (96, 90), (16, 40), (30, 30), (64, 70), (18, 18)]
    scenes, cfgs = [], []
    for nx, ny in sides:
        cfg = with_mode(W._base(grid_nx=nx, grid_ny=ny, grid_spacing=1.0 / (max(nx, ny) - 1), max_iterations=10,
                                shear_stiffness=900.0, bend_stiffness=20.0), "mixed")
        scenes.append(pdg.make_grid(cfg))
        cfgs.append(cfg)
    sim = pdg.Simulator(scenes, cfgs)
    sim.set_plan({"work_threads": threads})
    assert sim.plan()["work_threads"] == threads
    assert sim.info(0)["solve_kind"] == pdg.PD_SOLVE_SUPERNODAL32_CORRECTION
    for _ in range(12):
        sim.step(1)
    other = pdg.Simulator(scenes, cfgs)
    other.set_plan({"work_threads": threads})
    for _ in range(12):
        other.step(1)
    for i, (s, c) in enumerate(zip(scenes, cfgs)):
        assert np.array_equal(sim.state(i)[0].view(np.uint64), other.state(i)[0].view(np.uint64)), i
        orc = oracle_twin(s, c, perm=sim.factor(i)["perm"])
        orc.step(12)
        assert max_rel(sim.state(i)[0], orc.state()[0]) < TOL_POS, i
