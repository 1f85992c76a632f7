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
# FP32 solve; a cluster splitting the rows of the explicit FP32 inverse
STRATEGIES = {"one-cta": (1, 0), "cluster-supernodal": (16, -1), "cluster-dense": (16, 0)}


def with_mode(cfg, mode, ctas=0, dense=0):
    c = copy.copy(cfg)
    c.precision = MODES[mode]
    c.cluster_ctas = ctas
    c.dense_max_vertices = dense
    return c


def expected_kind(pdg, mode, ctas, dense):
    if MODES[mode] == pdg.PD_PRECISION_FP32_PROJECTION:
        return pdg.PD_SOLVE_SUPERNODAL
    return pdg.PD_SOLVE_DENSE32 if (ctas > 1 and dense >= 0) else pdg.PD_SOLVE_SUPERNODAL32


@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("strategy", list(STRATEGIES))
def test_plain_cloth_600_substeps(pdg, mode, strategy):
    scenes, cfg, substeps = W.cloth40_plain()
    ctas, dense = STRATEGIES[strategy]
    if MODES[mode] == pdg.PD_PRECISION_FP32_PROJECTION and strategy == "cluster-dense":
        pytest.skip("the FP64 solve has no dense variant")
    sim = pdg.Simulator(scenes[0], with_mode(cfg, mode, ctas, dense))
    assert sim.info()["solve_kind"] == expected_kind(pdg, mode, ctas, dense)
    orc = oracle_twin(scenes[0], cfg, perm=sim.factor()["perm"])
    sim.step(substeps)
    orc.step(substeps)
    err = max_rel(sim.state()[0], orc.state()[0])
    assert err < TOL_POS, err
    pins = np.flatnonzero(scenes[0].pinned)
    assert np.array_equal(sim.state()[0][pins], scenes[0].positions[pins])


@pytest.mark.parametrize("mode", ["mixed", "fp32-solve"])
@pytest.mark.parametrize("strategy", list(STRATEGIES))
def test_full_cloth_600_substeps(pdg, mode, strategy):
    scenes, cfg, substeps = W.cloth40_full()
    ctas, dense = STRATEGIES[strategy]
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
    """A 90×90 cloth does not fit the shared-memory workspace: one CTA with L2 workspaces."""
    cfg = with_mode(W._base(grid_nx=90, grid_ny=90, grid_spacing=1 / 89, max_iterations=10,
                            shear_stiffness=1000.0), "mixed")
    scene = pdg.make_grid(cfg)
    sim = pdg.Simulator(scene, cfg)
    assert sim.info()["solve_kind"] == pdg.PD_SOLVE_SUPERNODAL32
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    sim.step(30)
    orc.step(30)
    assert max_rel(sim.state()[0], orc.state()[0]) < TOL_POS
