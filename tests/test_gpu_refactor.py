"""Numeric refactorization on the GPU (refactor.cu): a stiffness or dt change keeps Ã's pattern,
so the LDLᵀ values, the block inverses and the FP32 copies are recomputed on the device. The new
factor against the host factorization of the changed scene (same ordering), and the simulation
after the change against the oracle making the same change; FP64_EXACT keeps the host factor.
"""
import copy
import os

import numpy as np
import pytest

from pd_gb300 import workloads as W
from pd_gb300.api import scene_factor
from tests.helpers import bits, max_rel, oracle_config, oracle_twin

pytestmark = pytest.mark.gpu

TOL = {1: 1e-10, 3: 1e-5, 4: 1e-5}


def cfg_with(cfg, precision, **kw):
    c = copy.copy(cfg)
    c.precision = precision
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def rel_err(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def changed(scene, k):
    s = copy.copy(scene)
    s.edge_stiffness = k
    return s


def check_stiffness_change(pdg, cfg, p, before=5, after=20):
    scene = pdg.make_grid(cfg)
    rng = np.random.default_rng(7)
    k2 = np.asarray(scene.edge_stiffness) * np.exp(rng.normal(0.0, 0.3, scene.edge_stiffness.shape))
    sim = pdg.Simulator(scene, cfg)
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    sim.step(before)
    orc.step(before)
    sim.set_edge_stiffness(k2)
    orc.set_edge_stiffness(k2)
    info = sim.info()
    assert info["factorize_count"] == 2 and info["device_factorize_count"] == 1
    # the device factor against the host factorization of the changed scene (same ordering)
    got = sim.factor()
    want, _ = scene_factor(changed(scene, k2), cfg)
    assert np.array_equal(got["perm"], want["perm"]) and np.array_equal(got["colptr"], want["colptr"])
    assert rel_err(got["val"], want["val"]) <= 1e-12 and rel_err(got["dinv"], want["dinv"]) <= 1e-12
    sim.step(after)
    orc.step(after)
    assert max_rel(sim.state()[0], orc.state()[0]) <= TOL[p]
    return sim


@pytest.mark.parametrize("p", [1, 3, 4])
def test_stiffness_change_small_cloth(pdg, p):
    cfg = cfg_with(W._base(grid_nx=24, grid_ny=20, grid_spacing=1 / 23, max_iterations=15, shear_stiffness=1000.0,
                           bend_stiffness=50.0), p)
    check_stiffness_change(pdg, cfg, p)


def test_stiffness_change_above_the_inverse_limit(pdg):
    """A MIXED cloth of 4480 vertices: the correction kernel's FP32 supernodal solve reads the new
    FP32 factor and block inverses."""
    cfg = cfg_with(W._base(grid_nx=70, grid_ny=64, grid_spacing=1 / 69, max_iterations=8, shear_stiffness=900.0), 4)
    sim = check_stiffness_change(pdg, cfg, 4, before=3, after=8)
    assert sim.info()["solve_kind"] == pdg.PD_SOLVE_SUPERNODAL32_CORRECTION


def test_dt_change(pdg):
    cfg = cfg_with(W._base(grid_nx=16, grid_ny=14, grid_spacing=1 / 15, max_iterations=10, shear_stiffness=800.0), 1)
    scene = pdg.make_grid(cfg)
    sim = pdg.Simulator(scene, cfg)
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    sim.step(4)
    orc.step(4)
    cfg2 = cfg_with(cfg, 1, dt=1.0 / 200.0)
    sim.set_config(cfg2)
    orc.set_config(oracle_config(cfg2))
    assert sim.info()["device_factorize_count"] == 1
    sim.step(12)
    orc.step(12)
    assert max_rel(sim.state()[0], orc.state()[0]) <= 1e-10


def test_reference_order_and_forced_host_path(pdg, monkeypatch):
    cfg = cfg_with(W._base(grid_nx=12, grid_ny=10, grid_spacing=0.05, max_iterations=8), 0)
    scene = pdg.make_grid(cfg)
    sim = pdg.Simulator(scene, cfg)
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    k2 = np.asarray(scene.edge_stiffness) * 1.3
    sim.set_edge_stiffness(k2)
    orc.set_edge_stiffness(k2)
    assert sim.info()["device_factorize_count"] == 0  # the host factor: bit parity
    sim.step(6)
    orc.step(6)
    assert np.array_equal(bits(sim.state()[0]), bits(orc.state()[0]))
    monkeypatch.setenv("PD_GB300_HOST_REFACTOR", "1")
    cfg1 = cfg_with(cfg, 1)
    sim1 = pdg.Simulator(scene, cfg1)
    sim1.set_edge_stiffness(k2)
    assert sim1.info()["device_factorize_count"] == 0 and sim1.info()["factorize_count"] == 2


@pytest.mark.parametrize("p", [0, 1, 4])
def test_failed_refactorization_keeps_the_handle(pdg, p):
    """A stiffness change whose Ã has a non-finite pivot (one edge of infinite stiffness) fails with
    PD_ERR_FACTORIZATION on the host path (reference order) and on the device path (the others);
    the handle keeps a whole factor, and after the stiffness is put back it steps like the oracle
    that never saw the change."""
    cfg = cfg_with(W._base(grid_nx=14, grid_ny=12, grid_spacing=1 / 13, max_iterations=8, shear_stiffness=700.0), p)
    scene = pdg.make_grid(cfg)
    sim = pdg.Simulator(scene, cfg)
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    sim.step(3)
    orc.step(3)
    k = np.asarray(scene.edge_stiffness, np.float64).copy()
    bad = k.copy()
    bad[len(bad) // 2] = np.inf
    with pytest.raises(pdg.PdError) as e:
        sim.set_edge_stiffness(bad)
    assert e.value.code == pdg.PD_ERR_FACTORIZATION
    sim.set_edge_stiffness(k)
    sim.step(6)
    orc.step(6)
    if p == 0:
        assert np.array_equal(bits(sim.state()[0]), bits(orc.state()[0]))
    else:
        assert max_rel(sim.state()[0], orc.state()[0]) <= TOL[p]
