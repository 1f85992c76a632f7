"""Failure detection of the team kernel without a GPU fault: every poll of an exchange is bounded
(2²² rounds, ~1–4 s), after which the CTA sets the instance's error flag and returns, and
pd_sim_synchronize reports PD_ERR_CUDA and resets the exchange words. A test hook makes one CTA
withhold its first exchange-A partial (a word nothing writes); the team's waits run out, the step
reports the error, and the same handle then steps exactly like a fresh one.
"""
import copy
import time

import numpy as np
import pytest

from pd_gb300 import workloads as W
from tests.helpers import bits

pytestmark = pytest.mark.gpu


def test_withheld_exchange_word_is_reported_and_the_handle_recovers(pdg, monkeypatch):
    cfg = copy.copy(W._base(grid_nx=20, grid_ny=18, grid_spacing=1 / 19, max_iterations=10, shear_stiffness=1000.0))
    cfg.precision = pdg.PD_PRECISION_MIXED
    scene = pdg.make_grid(cfg)
    x0, v0 = np.array(scene.positions), np.zeros((scene.n, 3))
    monkeypatch.setenv("PD_GB300_TEST_WITHHOLD_RANK", "3")
    sim = pdg.Simulator(scene, cfg)
    assert sim.info()["solve_kind"] == pdg.PD_SOLVE_DENSE32_TEAM and sim.info()["cluster_ctas"] > 3
    t0 = time.perf_counter()
    with pytest.raises(pdg.PdError) as e:
        sim.step(1)
    assert e.value.code == 4  # PD_ERR_CUDA: a team exchange gave up waiting
    assert time.perf_counter() - t0 < 120.0
    monkeypatch.delenv("PD_GB300_TEST_WITHHOLD_RANK")
    sim.set_residual_trace(False)  # rewrites the descriptors without the hook
    sim.set_state(0, x0, v0)
    sim.step(5)
    ref = pdg.Simulator(scene, cfg)
    ref.step(5)
    assert np.array_equal(bits(sim.state()[0]), bits(ref.state()[0]))
    assert np.array_equal(bits(sim.state()[1]), bits(ref.state()[1]))
