"""torch.autograd binding of the solve with respect to per-element log-coefficients.

    u = fem_solve(solver, theta, b, mask=None, lambda_mass=0.0)

assembles A(theta) = sum_e exp(theta_e) K_e + lambda_mass M on the solver's mesh,
eliminates the Dirichlet rows given by `mask`, builds the AMG hierarchy and solves
A u = b with the solver's PCG options.  Its backward pass is the adjoint solve of the
C ABI (femgpu_adjoint_grad): A lambda = dL/du with the same hierarchy, then
dL/dtheta_e = -exp(theta_e) lambda_e^T K_e u_e.  b is treated as a constant.

CUDA tensors stay on the device: the coefficients, b, u and the gradient pass through the
device entry points (femgpu_assemble_device, femgpu_solve_device,
femgpu_adjoint_grad_device); CPU tensors go through the host ones.  A forward or adjoint
solve that does not reach the tolerance raises.
"""
from __future__ import annotations

import numpy as np
import torch


def _status_error(what, st):
    return RuntimeError(f"{what} PCG did not converge: {st}")


class _FEMSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, solver, b, mask, lambda_mass):
        if theta.is_cuda:
            dev = theta.device
            coef = torch.exp(theta.detach().to(torch.float64)).contiguous()
            bb = b.detach().to(dev, torch.float64).contiguous()
            if mask is not None:
                m = torch.as_tensor(np.asarray(mask).astype(bool), device=dev)
                bb = torch.where(m, torch.zeros_like(bb), bb).contiguous()
            u = torch.zeros_like(bb)
            torch.cuda.synchronize(dev)  # the library's stream reads what torch's stream wrote
            solver.assemble_device(coef.data_ptr(), float(lambda_mass))
            if mask is not None:
                solver.set_dirichlet(mask)
            solver.setup()
            st = solver.solve_device(bb.data_ptr(), u.data_ptr(), check=False)
            if st["status"] != 0:
                raise _status_error("forward", st)
            ctx.solver = solver
            ctx.save_for_backward(u)
            return u
        th = theta.detach().to("cpu", torch.float64).numpy()
        solver.assemble(np.exp(th), float(lambda_mass))
        if mask is not None:
            solver.set_dirichlet(mask)
        solver.setup()
        bb = b.detach().to("cpu", torch.float64).numpy()
        if mask is not None:
            bb = np.where(np.asarray(mask).astype(bool), 0.0, bb)
        u, st = solver.solve(bb, check=False)
        if st["status"] != 0:
            raise _status_error("forward", st)
        ctx.solver = solver
        ut = torch.from_numpy(u)
        ctx.save_for_backward(ut)
        return ut

    @staticmethod
    def backward(ctx, grad_u):
        (u,) = ctx.saved_tensors
        if u.is_cuda:
            g = grad_u.detach().to(u.device, torch.float64).contiguous()
            grad = torch.empty(ctx.solver.nelems, dtype=torch.float64, device=u.device)
            torch.cuda.synchronize(u.device)
            st = ctx.solver.adjoint_grad_device(g.data_ptr(), u.data_ptr(), grad.data_ptr())
            if st["status"] != 0:
                raise _status_error("adjoint", st)
            return grad, None, None, None, None
        g = grad_u.detach().to("cpu", torch.float64).numpy()
        grad, st = ctx.solver.adjoint_grad(g, u.numpy(), check=False)
        if st["status"] != 0:
            raise _status_error("adjoint", st)
        return torch.from_numpy(grad), None, None, None, None


def fem_solve(solver, theta: torch.Tensor, b: torch.Tensor, mask=None, lambda_mass: float = 0.0) -> torch.Tensor:
    """Solve A(theta) u = b on `solver`'s mesh; differentiable in theta (see module doc)."""
    return _FEMSolve.apply(theta, solver, b, mask, lambda_mass)
