"""Differentiable static solve: a torch.autograd.Function over the C-ABI.

Forward: u = K'(E)^-1 f with per-element Young's moduli E (cfem_set_young +
cfem_pcg). Backward (hand-written adjoint, K' symmetric): lambda = K'^-1 dL/du
(second PCG solve, cfem_adjoint), then dL/dE_e = -lambda_e^T (dK'_e/dE_e) u_e
= -(1/E_e) lambda_e^T K'_e u_e (per-element kernel) and dL/df = lambda.

With CUDA tensors every array stays on the device: the library reads young, f,
u and dL/du and writes u, dL/dE and dL/df through device pointers, and the
context issues its work on the caller's current torch stream, so the solve is
ordered after whatever produced its inputs there. CPU tensors go through host
arrays instead.
"""
from __future__ import annotations

import numpy as np
import torch

from .solver import FemContext


def _f64(t: torch.Tensor) -> torch.Tensor:
    return t.detach().to(dtype=torch.float64).contiguous().view(-1)


class _StaticSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, young, f, fem: FemContext, precision: str, tol: float):
        kw = dict(precision=precision, tol=tol, stop_rule="residual", outer_tol=min(tol, 1e-12))
        if f.is_cuda:
            fem.set_stream(torch.cuda.current_stream(f.device))
            y, fb = _f64(young.to(f.device)), _f64(f)
            fem.set_young(y)
            u = torch.zeros_like(fb)
            fem.pcg(fb, out=u, **kw)
        else:
            fem.set_young(_f64(young).numpy())
            un, _ = fem.pcg(_f64(f).numpy(), **kw)
            u = torch.as_tensor(np.asarray(un), dtype=torch.float64)
        ctx.fem, ctx.precision, ctx.tol = fem, precision, tol
        ctx.save_for_backward(u)
        return u

    @staticmethod
    def backward(ctx, grad_u):
        (u,) = ctx.saved_tensors
        kw = dict(precision=ctx.precision, tol=ctx.tol, outer_tol=min(ctx.tol, 1e-12))
        g = _f64(grad_u)
        if u.is_cuda:
            ctx.fem.set_stream(torch.cuda.current_stream(u.device))
            gE, gf, _ = ctx.fem.adjoint(u, g.to(u.device), **kw)
        else:
            dE, df, _ = ctx.fem.adjoint(u.numpy(), g.numpy(), **kw)
            gE, gf = torch.as_tensor(dE), torch.as_tensor(df)
        return gE, gf, None, None, None


def static_solve(fem: FemContext, young: torch.Tensor, f: torch.Tensor, precision: str = "fp64",
                 tol: float = 1e-12) -> torch.Tensor:
    """u = K'(young)^-1 f, differentiable in ``young`` ([n_elems]) and ``f`` ([n_dof],
    caller node order). ``fem`` must be a context of the same mesh. CUDA
    tensors keep the solve and its adjoint on the device."""
    return _StaticSolve.apply(young, f, fem, precision, tol)
