"""Fitting and check harness for the differentiation form.

The gradients come from libsgmd.so's adjoint kernels (sg_diff_force_matching, through
engine.DiffModel); this module only carries them into torch: ForceMatchingLoss is a
torch.autograd.Function whose backward returns the library's gradient, so torch optimisers can
fit the 66 parameters (LJ epsilon, sigma and the two EAM splines, see include/sg_api.h).
"""
from __future__ import annotations

import numpy as np
import torch

from .engine import DiffModel


class ForceMatchingLoss(torch.autograd.Function):
    """loss = ForceMatchingLoss.apply(theta, model, ref_forces): theta a float64 tensor of 66
    parameters, model a DiffModel, ref_forces (N, 3) float32 numpy array."""

    @staticmethod
    def forward(ctx, theta: torch.Tensor, model: DiffModel, ref: np.ndarray) -> torch.Tensor:
        loss, grad = model.force_matching(theta.detach().cpu().double().numpy(), ref, grad=True)
        ctx.save_for_backward(torch.from_numpy(grad))
        return theta.new_tensor(loss)

    @staticmethod
    def backward(ctx, g: torch.Tensor):
        (grad,) = ctx.saved_tensors
        return g * grad.to(dtype=g.dtype, device=g.device), None, None


def fit(model: DiffModel, theta0: np.ndarray, ref: np.ndarray, steps: int = 50, lr: float = 1e-2):
    """Adam on relative changes of every parameter (theta = theta0 * (1 + x)); returns the fitted
    theta and the loss history."""
    base = torch.tensor(theta0, dtype=torch.float64)
    x = torch.zeros_like(base, requires_grad=True)
    opt = torch.optim.Adam([x], lr=lr)
    hist = []
    for _ in range(steps):
        opt.zero_grad()
        loss = ForceMatchingLoss.apply(base * (1 + x), model, ref)
        loss.backward()
        opt.step()
        hist.append(float(loss.detach()))
    return (base * (1 + x)).detach().numpy(), hist
