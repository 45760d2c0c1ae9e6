"""Differentiable static solve: a torch.autograd.Function over the C-ABI.

Forward: u = K'(E)^-1 f with per-element Young's moduli E (cfem_set_young +
cfem_pcg). Backward (hand-written adjoint, K' symmetric): lambda = K'^-1 dL/du
(second PCG solve, cfem_adjoint), then dL/dE_e = -lambda_e^T (dK'_e/dE_e) u_e
= -(1/E_e) lambda_e^T K'_e u_e (per-element kernel) and dL/df = lambda.
"""
from __future__ import annotations

import numpy as np
import torch

from .solver import FemContext


class _StaticSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, young, f, fem: FemContext, precision: str, tol: float):
        y = young.detach().double().cpu().numpy()
        fem.set_young(y)
        rule = "residual"
        u, _ = fem.pcg(f.detach().double().cpu().numpy(), precision=precision, tol=tol, stop_rule=rule,
                       outer_tol=min(tol, 1e-12))
        ut = torch.as_tensor(np.asarray(u), dtype=torch.float64, device=f.device)
        ctx.fem, ctx.precision, ctx.tol = fem, precision, tol
        ctx.save_for_backward(ut)
        return ut

    @staticmethod
    def backward(ctx, grad_u):
        (u,) = ctx.saved_tensors
        dE, df, _ = ctx.fem.adjoint(u.detach().cpu().numpy(), grad_u.detach().double().cpu().numpy(),
                                    precision=ctx.precision, tol=ctx.tol, outer_tol=min(ctx.tol, 1e-12))
        gE = torch.as_tensor(dE, dtype=torch.float64, device=grad_u.device)
        gf = torch.as_tensor(df, dtype=torch.float64, device=grad_u.device)
        return gE, gf, None, None, None


def static_solve(fem: FemContext, young: torch.Tensor, f: torch.Tensor, precision: str = "fp64",
                 tol: float = 1e-12) -> torch.Tensor:
    """u = K'(young)^-1 f, differentiable in ``young`` ([n_elems]) and ``f`` ([n_dof],
    caller node order). ``fem`` must be a context of the same mesh."""
    return _StaticSolve.apply(young, f, fem, precision, tol)
