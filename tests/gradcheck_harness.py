"""Gradient-check harness: the GPU adjoint (pd_sim_gradient) as a torch.autograd.Function.

Test infrastructure only: the product computes gradients through its C ABI and never depends on
torch's autograd; this wrapper lets torch.autograd.gradcheck and ordinary `loss.backward()` drive the
adjoint kernels, so the gradients are checked by torch's own finite-difference machinery.

PDRolloutLoss(kappa, v0, force) = mean over free vertices of |x_S − target|² after S substeps of
the cloth from its fixed initial positions, with per-edge stiffness `kappa`, initial velocities `v0`
and a constant external force `force` (float64 CPU tensors). The forward pass runs the substeps and
the adjoint on the GPU in one call; backward scales the stored gradients by the incoming gradient.
"""
from __future__ import annotations

import numpy as np
import torch


class RolloutProblem:
    """The fixed parts of the loss: simulator handle (one problem), substeps, targets, x₀."""

    def __init__(self, sim, substeps: int, targets, x0):
        self.sim = sim
        self.substeps = int(substeps)
        self.targets = np.ascontiguousarray(targets, np.float64)
        self.x0 = np.ascontiguousarray(x0, np.float64)
        self.evaluations = 0


class PDRolloutLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, kappa, v0, force, problem: RolloutProblem):
        sim = problem.sim
        sim.set_edge_stiffness(kappa.detach().cpu().numpy().astype(np.float64), 0)
        sim.set_state(0, problem.x0, v0.detach().cpu().numpy().reshape(-1, 3))
        want = any(ctx.needs_input_grad[:3])
        out = sim.gradient(problem.substeps, problem.targets, force.detach().cpu().numpy().reshape(-1, 3), grad=want)
        problem.evaluations += 1
        if want:
            ctx.save_for_backward(torch.from_numpy(out["dkappa"].copy()),
                                  torch.from_numpy(out["dv0"].reshape(v0.shape).copy()),
                                  torch.from_numpy(out["dforce"].reshape(force.shape).copy()))
        return torch.tensor(out["loss"], dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad_out):
        dk, dv, df = ctx.saved_tensors
        return grad_out * dk, grad_out * dv, grad_out * df, None


def rollout_loss(kappa, v0, force, problem: RolloutProblem):
    return PDRolloutLoss.apply(kappa, v0, force, problem)
