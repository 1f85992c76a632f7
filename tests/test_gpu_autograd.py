"""The adjoint kernels behind torch.autograd (tests/gradcheck_harness.py): torch's gradcheck on the
rollout loss (its central differences along random directions, in float64), backward() returning
exactly the kernels' gradients, and a few steps of gradient descent on the stiffness recovering part
of a hidden stiffness field.
"""
import copy

import numpy as np
import pytest
import torch

from pd_gb300 import workloads as W
from tests.gradcheck_harness import RolloutProblem, rollout_loss
from tests.helpers import oracle_twin

pytestmark = pytest.mark.gpu


def _problem(pdg, side=8, substeps=6):
    scene, cfg, S, kstar = W.differentiable(side=side, substeps=substeps)
    c = copy.copy(cfg)
    c.precision = 1
    twin = oracle_twin(scene, c)
    twin.set_edge_stiffness(kstar)
    twin.step(S)
    sim = pdg.Simulator(scene, c)
    return scene, RolloutProblem(sim, S, twin.state()[0], scene.positions), kstar


def _params(scene, seed=0):
    rng = np.random.default_rng(seed)
    kappa = torch.tensor(np.asarray(scene.edge_stiffness, np.float64) * (1.0 + 0.05 * rng.standard_normal(
        scene.edges.shape[0])), dtype=torch.float64, requires_grad=True)
    v0 = np.zeros((scene.n, 3))
    v0[np.flatnonzero(scene.pinned == 0)] = 0.02 * rng.standard_normal((int(np.sum(scene.pinned == 0)), 3))
    v0 = torch.tensor(v0, requires_grad=True)
    force = torch.tensor(0.01 * rng.standard_normal((scene.n, 3)), requires_grad=True)
    return kappa, v0, force


def test_torch_gradcheck_on_the_rollout_loss(pdg):
    """torch.autograd.gradcheck (fast mode: central differences along random directions against the
    backward pass) on the loss normalised by its value at the start. The checked variables are
    displacements in scaled units, 100 × (stiffness relative to itself, velocity in m/s, force in
    vertex weights), so that the step eps = 1e-6 moves each parameter by ~1e-4 of its scale: a
    smaller step would only measure the rounding of the loss (every stiffness step refactorizes L,
    and the loss is a small difference of positions), a larger one the curvature."""
    scene, prob, _ = _problem(pdg)
    kappa, v0, force = _params(scene)
    k0, v00, f0 = kappa.detach().clone(), v0.detach().clone(), force.detach().clone()
    weight = torch.tensor(np.asarray(scene.masses, np.float64)[:, None] * 9.81)
    loss0 = rollout_loss(k0, v00, f0, prob).item()
    assert loss0 > 0.0
    sk = torch.zeros_like(k0, requires_grad=True)
    sv = torch.zeros_like(v00, requires_grad=True)
    sf = torch.zeros_like(f0, requires_grad=True)

    def f(sk_, sv_, sf_):
        return rollout_loss(k0 * (1.0 + 100.0 * sk_), v00 + 100.0 * sv_, f0 + weight * (100.0 * sf_), prob) / loss0

    ok = torch.autograd.gradcheck(f, (sk, sv, sf), eps=1e-6, atol=1e-8, rtol=1e-5, fast_mode=True)
    assert ok and prob.evaluations > 3


def test_backward_returns_the_adjoint_kernels_gradients(pdg):
    scene, prob, _ = _problem(pdg)
    kappa, v0, force = _params(scene, seed=1)
    loss = rollout_loss(kappa, v0, force, prob)
    loss.backward()
    sim = prob.sim
    sim.set_edge_stiffness(kappa.detach().numpy(), 0)
    sim.set_state(0, prob.x0, v0.detach().numpy())
    g = sim.gradient(prob.substeps, prob.targets, force.detach().numpy())
    assert loss.item() == g["loss"]
    assert np.array_equal(kappa.grad.numpy(), g["dkappa"])
    assert np.array_equal(v0.grad.numpy(), g["dv0"].reshape(v0.shape))
    assert np.array_equal(force.grad.numpy(), g["dforce"].reshape(force.shape))


def test_gradient_descent_on_stiffness_lowers_the_loss(pdg):
    """Log-stiffness descent with torch's optimiser, gradients from the adjoint kernels."""
    scene, prob, kstar = _problem(pdg, side=10, substeps=10)
    logk = torch.tensor(np.log(np.asarray(scene.edge_stiffness, np.float64)), requires_grad=True)
    v0 = torch.zeros((scene.n, 3), dtype=torch.float64)
    force = torch.zeros((scene.n, 3), dtype=torch.float64)
    opt = torch.optim.Adam([logk], lr=0.02)
    losses = []
    for _ in range(12):
        opt.zero_grad()
        loss = rollout_loss(torch.exp(logk), v0, force, prob)
        loss.backward()
        opt.step()
        losses.append(loss.item())
    assert losses[1] < losses[0] and losses[-1] < losses[0], losses
