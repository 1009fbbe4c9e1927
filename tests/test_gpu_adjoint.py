"""Adjoint gradient of the solve w.r.t. per-element log-coefficients (needs a GB300).

The GPU gradient (femgpu_adjoint_grad: adjoint PCG with the forward hierarchy plus the
element kernel) is checked against the FP64 reference gradient (scipy direct solves,
numpy element restatement) and against central differences with h = 1e-6.
"""
import numpy as np
import pytest

import adjoint_ref as R
import femgpu

pytestmark = pytest.mark.gpu


def gpu_forward(xyz, conn, theta, mask, b, precision):
    s = femgpu.Solver(solverType=1, tolerance=1e-12, maxIters=1000, flexibleCG=1, seed=3, precision=precision)
    s.set_mesh(xyz, conn)
    s.assemble(np.exp(theta), 0.0)
    s.set_dirichlet(mask)
    s.setup()
    u, st = s.solve(np.where(mask.astype(bool), 0.0, b))
    assert st["status"] == 0
    return s, u


@pytest.mark.parametrize("dim,n,precision", [(3, 10, 0), (3, 10, 1), (2, 24, 0)])
def test_adjoint_gradient_matches_fp64_reference(dim, n, precision):
    xyz, conn, theta, mask, b, S, u_obs = R.problem(n, dim=dim)
    s, u = gpu_forward(xyz, conn, theta, mask, b, precision)
    u_ref = R.solve(xyz, conn, theta, mask, b)
    assert np.linalg.norm(u - u_ref) / np.linalg.norm(u_ref) < 1e-9
    L, dLdu = R.loss_and_dLdu(u, S, u_obs)
    g, st = s.adjoint_grad(dLdu, u)
    assert st["status"] == 0 and st["relres"] <= 1e-12
    g_ref = R.gradient(xyz, conn, theta, mask, dLdu, u)
    rel = np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref)
    assert rel < 1e-8, rel


def test_adjoint_gradient_matches_central_differences():
    xyz, conn, theta, mask, b, S, u_obs = R.problem(8, dim=3)
    s, u = gpu_forward(xyz, conn, theta, mask, b, 0)
    L, dLdu = R.loss_and_dLdu(u, S, u_obs)
    g, _ = s.adjoint_grad(dLdu, u)
    rng = np.random.default_rng(12)
    h = 1e-6
    elems = rng.choice(conn.shape[0], 32, replace=False)
    fd = np.zeros(len(elems))
    for q, e in enumerate(elems):
        tp, tm = theta.copy(), theta.copy()
        tp[e] += h
        tm[e] -= h
        Lp, _ = R.loss_and_dLdu(R.solve(xyz, conn, tp, mask, b), S, u_obs)
        Lm, _ = R.loss_and_dLdu(R.solve(xyz, conn, tm, mask, b), S, u_obs)
        fd[q] = (Lp - Lm) / (2 * h)
    rel = np.linalg.norm(fd - g[elems]) / np.linalg.norm(g[elems])
    assert rel <= 1e-6, rel


@pytest.mark.parametrize("device", ["cpu", "cuda"])
def test_torch_autograd_binding(device):
    # CUDA tensors stay on the device (device entry points), CPU tensors go through the host
    torch = pytest.importorskip("torch")
    from femgpu.autograd import fem_solve

    xyz, conn, theta, mask, b, S, u_obs = R.problem(8, dim=3)
    s = femgpu.Solver(solverType=1, tolerance=1e-12, maxIters=1000, flexibleCG=1, seed=3)
    s.set_mesh(xyz, conn)
    th = torch.tensor(theta, dtype=torch.float64, device=device, requires_grad=True)
    u = fem_solve(s, th, torch.from_numpy(b).to(device), mask=mask)
    assert u.device.type == device
    Si = torch.from_numpy(S).to(device)
    loss = 0.5 * ((u[Si] - torch.from_numpy(u_obs).to(device)[Si]) ** 2).sum()
    loss.backward()
    assert th.grad.device.type == device
    u_np = u.detach().cpu().numpy()
    _, dLdu = R.loss_and_dLdu(u_np, S, u_obs)
    g_ref = R.gradient(xyz, conn, theta, mask, dLdu, u_np)
    rel = np.linalg.norm(th.grad.cpu().numpy() - g_ref) / np.linalg.norm(g_ref)
    assert rel < 1e-8, rel


def test_adjoint_needs_mesh_assembly():
    xyz, conn, theta, mask, b, S, u_obs = R.problem(4, dim=3)
    s = femgpu.Solver(solverType=1)
    s.set_mesh(xyz, conn)
    A = R.operator(xyz, conn, theta, mask).tocsr()
    s.set_matrix_csr(A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data)
    with pytest.raises(femgpu.FemgpuError):
        s.adjoint_grad(np.ones(xyz.shape[0]), np.ones(xyz.shape[0]))


def test_torch_binding_raises_when_the_solve_fails():
    torch = pytest.importorskip("torch")
    from femgpu.autograd import fem_solve

    xyz, conn, theta, mask, b, S, u_obs = R.problem(8, dim=3)
    s = femgpu.Solver(solverType=1, tolerance=1e-14, maxIters=2, flexibleCG=1, seed=3)
    s.set_mesh(xyz, conn)
    th = torch.tensor(theta, dtype=torch.float64, device="cuda", requires_grad=True)
    with pytest.raises(RuntimeError, match="forward PCG"):
        fem_solve(s, th, torch.from_numpy(b).cuda(), mask=mask)
