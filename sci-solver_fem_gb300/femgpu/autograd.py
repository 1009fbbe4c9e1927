"""torch.autograd binding of the solve with respect to per-element log-coefficients.

    u = fem_solve(solver, theta, b, mask=None, lambda_mass=0.0)

assembles A(theta) = sum_e exp(theta_e) K_e + lambda_mass M on the solver's mesh,
eliminates the Dirichlet rows given by `mask`, builds the AMG hierarchy and solves
A u = b with the solver's PCG options.  Its backward pass is the adjoint solve of the
C ABI (femgpu_adjoint_grad): A lambda = dL/du with the same hierarchy, then
dL/dtheta_e = -exp(theta_e) lambda_e^T K_e u_e.  b is treated as a constant.

The tensors may live on the CPU or the GPU; the solver copies through the C ABI.
"""
from __future__ import annotations

import numpy as np
import torch


class _FEMSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, solver, b, mask, lambda_mass):
        th = theta.detach().to("cpu", torch.float64).numpy()
        solver.assemble(np.exp(th), float(lambda_mass))
        if mask is not None:
            solver.set_dirichlet(mask)
        solver.setup()
        bb = b.detach().to("cpu", torch.float64).numpy()
        if mask is not None:
            bb = np.where(np.asarray(mask).astype(bool), 0.0, bb)
        u, st = solver.solve(bb)
        if st["status"] != 0:
            raise RuntimeError(f"forward PCG did not converge: {st}")
        ctx.solver = solver
        ctx.u = u
        ctx.device = theta.device
        return torch.from_numpy(u).to(theta.device)

    @staticmethod
    def backward(ctx, grad_u):
        g = grad_u.detach().to("cpu", torch.float64).numpy()
        grad, st = ctx.solver.adjoint_grad(g, ctx.u)
        return torch.from_numpy(grad).to(ctx.device), None, None, None, None


def fem_solve(solver, theta: torch.Tensor, b: torch.Tensor, mask=None, lambda_mass: float = 0.0) -> torch.Tensor:
    """Solve A(theta) u = b on `solver`'s mesh; differentiable in theta (see module doc)."""
    return _FEMSolve.apply(theta, solver, b, mask, lambda_mass)
