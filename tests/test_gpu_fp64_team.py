"""The FP64 team kernel (PD_SOLVE_DENSE64_TEAM): PD_PRECISION_FP64 on small cloths, the correction
form against the explicit inverse with the product in double-float arithmetic, held to the FP64 bar
against the oracle — positions within 1e-10 relative after the full 600-substep scenes and the
same per-substep iteration counts (the gate decides alike) — with the residual and displacement
gates, pin drags, batches sharing the SMs, repeated launches and other team sizes, and a withheld
exchange word reported without a fault.
"""
import copy
import time

import numpy as np
import pytest

from pd_gb300 import workloads as W
from tests.helpers import bits, max_rel, oracle_twin

pytestmark = pytest.mark.gpu

TOL_POS = 1e-10


def fp64(cfg, **kw):
    c = copy.copy(cfg)
    c.precision = 1
    for k, v in kw.items():
        setattr(c, k, v)
    return c


@pytest.mark.parametrize("name", ["cloth40_plain", "cloth40_full"])
def test_600_substeps_within_fp64_bar(pdg, name):
    scenes, cfg, substeps = W.WORKLOADS[name]()
    sim = pdg.Simulator(scenes[0], fp64(cfg))
    info = sim.info()
    assert info["solve_kind"] == pdg.PD_SOLVE_DENSE64_TEAM and info["cluster_ctas"] > 16
    orc = oracle_twin(scenes[0], cfg, perm=sim.factor()["perm"])
    sim.step(substeps)
    it_o, _ = orc.step(substeps)
    assert np.array_equal(sim.iteration_log()[0], it_o)
    xg, vg = sim.state()
    xo, vo = orc.state()
    assert max_rel(xg, xo) < TOL_POS, max_rel(xg, xo)
    assert max_rel(vg, vo) < 1e-7
    pins = np.flatnonzero(scenes[0].pinned)
    assert np.array_equal(xg[pins], scenes[0].positions[pins])


@pytest.mark.parametrize("gate", ["residual", "displacement"])
def test_gates_decide_like_the_oracle(pdg, gate):
    kw = {"residual": dict(residual_tolerance=0.3), "displacement": dict(residual_tolerance=0.0, rel_tolerance=2e-2)}
    cfg = fp64(W._base(grid_nx=14, grid_ny=12, grid_spacing=0.05, max_iterations=30, velocity_damping=0.02,
                       shear_stiffness=800.0, bend_stiffness=20.0, **kw[gate]))
    scene = pdg.make_grid(cfg)
    sim = pdg.Simulator(scene, cfg)
    assert sim.info()["solve_kind"] == pdg.PD_SOLVE_DENSE64_TEAM
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    sim.step(150)
    it_o, _ = orc.step(150)
    it_g, _ = sim.iteration_log()
    assert np.array_equal(it_g, it_o) and it_o.min() < 30
    assert max_rel(sim.state()[0], orc.state()[0]) < TOL_POS
    if gate == "residual":
        assert sim.stats()["last_residual"] == pytest.approx(orc.stats()["last_residual"], rel=1e-9)


def test_pin_drags_and_repeated_launches(pdg):
    scenes, cfg, _ = W.cloth40_full()
    scene = scenes[0]
    sim = pdg.Simulator(scene, fp64(cfg))
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    q = np.array(scene.positions)
    pins = np.flatnonzero(scene.pinned)
    for r in range(4):
        q[pins, 1] += 0.01
        q[pins, 0] -= 0.005 * r
        sim.set_pin_positions(q)
        orc.set_pin_positions(q)
        for _ in range(5):  # one substep per launch: the exchange epochs carry over
            sim.step(1)
        orc.step(5)
    xg = sim.state()[0]
    assert max_rel(xg, orc.state()[0]) < TOL_POS
    assert np.array_equal(xg[pins], q[pins])


def test_batch_shares_the_sms(pdg):
    scenes, cfgs, _ = W.batch(count=6, seed=21, max_side=40)
    cfgs = [fp64(c) for c in cfgs]
    sim = pdg.Simulator(scenes, cfgs)
    assert sim.info(0)["solve_kind"] == pdg.PD_SOLVE_DENSE64_TEAM and sim.info(0)["cluster_ctas"] == 152 // 6
    sim.step(40)
    for i, (s, c) in enumerate(zip(scenes, cfgs)):
        orc = oracle_twin(s, c, perm=sim.factor(i)["perm"])
        it_o, _ = orc.step(40)
        assert np.array_equal(sim.iteration_log(i)[0], it_o), i
        assert max_rel(sim.state(i)[0], orc.state()[0]) < TOL_POS, i


@pytest.mark.parametrize("team", [17, 40, 151])
def test_team_sizes(pdg, team):
    """Other team sizes (a plan's team_ctas above 16: 16 or fewer asks for the supernodal cluster)
    split the rows of Ã⁻¹ differently: each stays within the FP64 bar."""
    scenes, cfg, _ = W.cloth40_plain()
    sim = pdg.Simulator(scenes[0], fp64(cfg))
    sim.set_plan({"team_ctas": team})
    assert sim.info()["solve_kind"] == pdg.PD_SOLVE_DENSE64_TEAM and sim.info()["cluster_ctas"] == team
    orc = oracle_twin(scenes[0], cfg, perm=sim.factor()["perm"])
    sim.step(120)
    it_o, _ = orc.step(120)
    assert np.array_equal(sim.iteration_log()[0], it_o)
    assert max_rel(sim.state()[0], orc.state()[0]) < TOL_POS


def test_cluster_request_and_no_dense_keep_the_supernodal_kernel(pdg):
    scenes, cfg, _ = W.cloth40_plain()
    assert pdg.Simulator(scenes[0], fp64(cfg, cluster_ctas=16)).info()["solve_kind"] == pdg.PD_SOLVE_SUPERNODAL
    assert pdg.Simulator(scenes[0], fp64(cfg, dense_max_vertices=-1)).info()["solve_kind"] == pdg.PD_SOLVE_SUPERNODAL
    cheb = fp64(cfg, cheb_mode=pdg.PD_CHEB_RHO)
    assert pdg.Simulator(scenes[0], cheb).info()["solve_kind"] == pdg.PD_SOLVE_SUPERNODAL


def test_host_state_steps_like_device_state(pdg):
    scenes, cfg, _ = W.cloth40_full()
    a = pdg.Simulator(scenes[0], fp64(cfg))
    b = pdg.Simulator(scenes[0], fp64(cfg))
    import torch
    x0, v0 = b.state()
    hx = torch.from_numpy(x0.copy()).pin_memory()
    hv = torch.from_numpy(v0.copy()).pin_memory()
    b.bind_host([hx.numpy()], [hv.numpy()])
    for _ in range(3):
        a.step(4)
        b.step_host(4)
    assert np.array_equal(bits(hx.numpy()), bits(a.state()[0]))
    assert np.array_equal(bits(hv.numpy()), bits(a.state()[1]))


def test_withheld_exchange_word_is_reported_and_the_handle_recovers(pdg, monkeypatch):
    cfg = fp64(W._base(grid_nx=20, grid_ny=18, grid_spacing=1 / 19, max_iterations=10, shear_stiffness=1000.0))
    scene = pdg.make_grid(cfg)
    x0, v0 = np.array(scene.positions), np.zeros((scene.n, 3))
    monkeypatch.setenv("PD_GB300_TEST_WITHHOLD_RANK", "5")
    sim = pdg.Simulator(scene, cfg)
    assert sim.info()["solve_kind"] == pdg.PD_SOLVE_DENSE64_TEAM and sim.info()["cluster_ctas"] > 5
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
