"""Per-iteration residual trace (pd_sim_set_residual_trace) against the oracle's gate residuals:
bit-identical in the reference-order FP64 mode, close in the FP32 modes, NaN past early exits."""
import copy

import numpy as np
import pytest

from pd_gb300 import workloads as W
from tests.helpers import oracle_twin

pytestmark = pytest.mark.gpu


def test_reference_order_trace_bit_identical(pdg):
    cfg = W._base(grid_nx=12, grid_ny=12, grid_spacing=0.05, max_iterations=30, residual_tolerance=0.3,
                  velocity_damping=0.02)
    scene = pdg.make_grid(cfg)
    sim = pdg.Simulator(scene, cfg)
    sim.set_residual_trace(True)
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    sim.step(25)
    tg = sim.residual_trace()
    to = orc.step_traced(25)
    assert tg.shape == to.shape == (25, 30)
    assert np.array_equal(np.isnan(tg), np.isnan(to)) and np.isnan(tg).any()  # the gate fires
    m = ~np.isnan(to)
    assert np.array_equal(tg[m].view(np.uint64), to[m].view(np.uint64))
    it, _ = sim.iteration_log()
    assert np.array_equal((~np.isnan(tg)).sum(axis=1), it)


@pytest.mark.parametrize("precision,ctas", [(1, 16), (4, 0), (4, 1), (3, 1)])
def test_fast_mode_traces(pdg, precision, ctas):
    scenes, cfg, _ = W.cloth40_full()
    c = copy.copy(cfg)
    c.precision = precision
    c.cluster_ctas = ctas
    sim = pdg.Simulator(scenes[0], c)
    sim.set_residual_trace(True)
    orc = oracle_twin(scenes[0], cfg, perm=sim.factor()["perm"])
    sim.step(8)
    tg = sim.residual_trace()
    to = orc.step_traced(8)
    assert not np.isnan(to).any() and not np.isnan(tg).any()  # 40 iterations, gate never met
    rel = np.max(np.abs(tg - to) / to)
    assert rel < (1e-8 if precision == 1 else 2e-2), rel
    sim.set_residual_trace(False)
    sim.step(1)
    with pytest.raises(pdg.PdError):
        sim.residual_trace()
