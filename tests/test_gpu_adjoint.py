"""Adjoint gradients on the GPU (pd_sim_gradient) against the FP64 CPU reference gradient and
central finite differences of the GPU's own loss.

Problem: the differentiable workload (grid cloth, distance + shear edges at κ = 2300, gate off);
targets are the final positions of an oracle run with the hidden per-edge stiffness κ*; a seeded
external force. Gradients w.r.t. per-edge κ, initial velocities and the force.
"""
import copy

import numpy as np
import pytest

from pd_gb300 import workloads as W
from tests.helpers import oracle_twin

pytestmark = pytest.mark.gpu


def problem(side=12, substeps=15, seed=7):
    scene, cfg, S, kstar = W.differentiable(side=side, substeps=substeps)
    twin = oracle_twin(scene, cfg)
    twin.set_edge_stiffness(kstar)
    twin.step(S)
    targets = twin.state()[0]
    rng = np.random.default_rng(seed)
    force = rng.normal(0.0, 0.05, (scene.n, 3))
    v0 = rng.normal(0.0, 0.05, (scene.n, 3))
    v0[np.flatnonzero(scene.pinned)] = 0.0
    c = copy.copy(cfg)
    c.precision = 1  # FP64
    return scene, c, S, targets, force, v0, rng


def rel_norm(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


def test_gradient_matches_cpu_reference(pdg):
    scene, cfg, S, targets, force, v0, _ = problem()
    sim = pdg.Simulator(scene, cfg)
    x0 = sim.state()[0]
    sim.set_state(0, x0, v0)
    g = sim.gradient(S, targets, force)
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    orc.set_state(x0, v0)
    r = orc.gradient(S, targets, force)
    assert abs(g["loss"] - r["loss"]) <= 1e-10 * r["loss"]
    for key in ("dkappa", "dv0", "dforce"):
        assert rel_norm(g[key], r[key]) < 1e-8, key
    # the state is left unchanged
    x1, v1 = sim.state()
    assert np.array_equal(x1, x0) and np.array_equal(v1, v0)


def test_gradient_matches_central_differences(pdg):
    """Directional derivatives against central differences of the GPU loss, all evaluations in
    one batched launch (2 per direction, loss only)."""
    scene, cfg, S, targets, force, v0, rng = problem()
    sim = pdg.Simulator(scene, cfg)
    x0 = sim.state()[0]
    sim.set_state(0, x0, v0)
    g = sim.gradient(S, targets, force)
    k0 = np.asarray(scene.edge_stiffness, np.float64)
    eps, dirs = 1e-4, 4
    D = [(k0 * rng.normal(0.0, 0.05, k0.shape), rng.normal(0.0, 0.1, v0.shape), rng.normal(0.0, 0.05, force.shape))
         for _ in range(dirs)]
    batch = pdg.Simulator([scene] * (2 * dirs), [cfg] * (2 * dirs))
    forces = []
    for j, (dk, dv, df) in enumerate(D):
        for s, sign in enumerate((1.0, -1.0)):
            i = 2 * j + s
            batch.set_edge_stiffness(k0 + sign * eps * dk, i)
            batch.set_state(i, x0, v0 + sign * eps * dv)
            forces.append(force + sign * eps * df)
    losses = batch.gradient(S, [targets] * (2 * dirs), forces, grad=False)
    for j, (dk, dv, df) in enumerate(D):
        fd = (losses[2 * j]["loss"] - losses[2 * j + 1]["loss"]) / (2 * eps)
        adj = g["dkappa"] @ dk + np.sum(g["dv0"] * dv) + np.sum(g["dforce"] * df)
        assert abs(fd - adj) <= 1e-6 * abs(adj), (j, fd, adj)


def test_gradient_batch_equals_single_problems(pdg):
    scene, cfg, S, targets, force, v0, rng = problem(side=10, substeps=8)
    forces = [force, 2.0 * force, None]
    batch = pdg.Simulator([scene] * 3, [cfg] * 3)
    for i in range(3):
        batch.set_state(i, scene.positions, v0)
    gb = batch.gradient(S, [targets] * 3, forces)
    for i in range(3):
        one = pdg.Simulator(scene, cfg)
        one.set_state(0, scene.positions, v0)
        g1 = one.gradient(S, targets, forces[i])
        assert gb[i]["loss"] == g1["loss"]
        for key in ("dkappa", "dv0", "dforce"):
            assert np.array_equal(gb[i][key], g1[key]), (i, key)


def test_stored_iterates_equal_recomputed(pdg, monkeypatch):
    """The reverse pass reads every stored iterate, or recomputes each substep from its checkpoint
    when the store is capped to zero: the same gradient bit for bit."""
    scene, cfg, S, targets, force, v0, _ = problem(side=10, substeps=8)
    out = []
    for cap in (None, "0"):
        if cap is None:
            monkeypatch.delenv("PD_GB300_GRADIENT_STORE_BYTES", raising=False)
        else:
            monkeypatch.setenv("PD_GB300_GRADIENT_STORE_BYTES", cap)
        sim = pdg.Simulator(scene, cfg)
        sim.set_state(0, scene.positions, v0)
        out.append(sim.gradient(S, targets, force))
    assert out[0]["loss"] == out[1]["loss"]
    for key in ("dkappa", "dv0", "dforce"):
        assert np.array_equal(out[0][key], out[1][key]), key
