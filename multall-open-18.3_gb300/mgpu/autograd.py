"""torch.autograd wrapper of the adjoint gradient, for check harnesses.

`DesignSolve` marches a design's deck to convergence on the GPU and returns
an objective with its gradient with respect to the blade-angle design
variables (mgpu_adjoint_* plus the chain in design.py).  `AdjointObjective`
exposes that as a differentiable function of a torch tensor of design
variables, so a harness can call `.backward()` or hand it to an optimiser.
torch is plumbing here: the values and gradients come from the C ABI.
"""
from __future__ import annotations

import numpy as np
import torch

from . import design as _design
from . import lib as _lib


class DesignSolve:
    """Primal solve plus adjoint gradient of one objective for a design."""

    def __init__(self, space: _design.DesignSpace, steps: int = 3000, adjoint_iters: int = 8000,
                 krylov: bool = False):
        self.space = space
        self.steps = steps
        self.adjoint_iters = adjoint_iters
        self.krylov = krylov
        self.last = None

    def value_and_gradient(self, alpha: np.ndarray, objective: str):
        cd = self.space.deck(alpha)
        cd.ints["NSTEPS_MAX"] = 10 ** 9
        cd.reals["CONLIM"] = 1e-9
        p = _lib.Problem(cd)
        try:
            p.run(self.steps)
            p.adjoint_prepare()
            value = p.adjoint_objective(objective)
            if self.krylov:
                p.adjoint_solve_krylov(max_steps=self.adjoint_iters)
            else:
                p.adjoint_iterate(self.adjoint_iters)
            grad = self.space.chain(p.adjoint_gradient(), self.space.sensitivities(alpha))
        finally:
            p.close()
        self.last = (value, grad)
        return value, grad


class AdjointObjective(torch.autograd.Function):
    """J(alpha) with dJ/dalpha from the discrete adjoint."""

    @staticmethod
    def forward(ctx, alpha: torch.Tensor, solver: DesignSolve, objective: str):
        value, grad = solver.value_and_gradient(alpha.detach().cpu().double().numpy(), objective)
        ctx.save_for_backward(torch.as_tensor(grad, dtype=alpha.dtype, device=alpha.device))
        return alpha.new_tensor(value)

    @staticmethod
    def backward(ctx, g):
        (grad,) = ctx.saved_tensors
        return g * grad, None, None
