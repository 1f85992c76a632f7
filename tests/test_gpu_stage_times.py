"""StageTimes on the device (pd_sim_set_stage_timing): per-stage seconds that partition each
substep's total, for the reference-order kernel, the FP64 cluster kernel, the MIXED team kernel and
the correction kernel; off by default, reset by resetStageTimes, `assemble` from refactorizations.
"""
import copy

import numpy as np
import pytest
import torch

from pd_gb300 import workloads as W

pytestmark = pytest.mark.gpu

DEVICE = ("predict", "local_step", "scatter", "solve", "unpack_scan", "velocity")


@pytest.mark.parametrize("p,side", [(0, 12), (1, 30), (4, 24), (4, 70)])
def test_stages_partition_the_substep(pdg, p, side):
    cfg = copy.copy(W._base(grid_nx=side, grid_ny=side, grid_spacing=1 / (side - 1), max_iterations=8,
                            shear_stiffness=900.0, bend_stiffness=30.0))
    cfg.precision = p
    sim = pdg.Simulator(pdg.make_grid(cfg), cfg)
    sim.step(2)
    assert all(v == 0.0 for k, v in sim.stage_times().items() if k != "assemble")  # off by default
    sim.set_stage_timing(True)
    stream = torch.cuda.Stream()
    sim.set_stream(stream.cuda_stream)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    sim.step(5, sync=False)
    b.record(stream)
    sim.synchronize()
    launch_s = a.elapsed_time(b) * 1e-3
    t = sim.stage_times()
    for k in ("predict", "local_step", "solve", "unpack_scan", "velocity"):
        assert t[k] > 0.0, (k, t)
    assert sum(t[k] for k in DEVICE) == pytest.approx(t["total"], rel=1e-9)
    assert 0.3 * launch_s <= t["total"] <= 1.05 * launch_s, (t["total"], launch_s)
    assert t["assemble"] > 0.0  # the creation's factorization
    sim.reset_stage_times()
    assert all(v == 0.0 for v in sim.stage_times().values())
    sim.set_edge_stiffness(np.asarray(pdg.make_grid(cfg).edge_stiffness) * 1.1)
    assert sim.stage_times()["assemble"] > 0.0
