"""The differentiation configuration at full size (needs a GB300): 96^3 Kuhn mesh (912,673
vertices, 5,308,416 tets), theta_e = log kappa_e ~ N(0,1) (seed 9), f ~ U[-1,1] (seed 5),
u = 0 on z = 0, loss 0.5 ||u[S] - u_obs||^2 over a seeded 1% vertex set S (seed 10) with
u_obs from a second theta (seed 11).

The mixed-precision gradient (FP32 hierarchy, forward and adjoint PCG to 1e-10) is checked
against the FP64-hierarchy gradient solved to 1e-12 (<= 1e-6 relative), and against central
differences with h = 1e-6 on 32 seeded elements (seed 12, <= 1e-6 relative)."""
import numpy as np
import pytest

import femgpu
from femgpu import gradcheck, meshes

pytestmark = pytest.mark.gpu


def forward(xyz, conn, theta, mask, f, precision, tol):
    s = femgpu.Solver(solverType=1, tolerance=tol, maxIters=3000, flexibleCG=1, seed=1, precision=precision)
    s.set_mesh(xyz, conn)
    b = np.where(mask.astype(bool), 0.0, s.load_vector(f))
    s.assemble(np.exp(theta), 0.0)
    s.set_dirichlet(mask)
    s.setup()
    u, st = s.solve(b)
    assert st["status"] == 0
    return s, u, b


@pytest.fixture(scope="module")
def problem():
    xyz, conn = meshes.kuhn_cube(96)
    n, ne = xyz.shape[0], conn.shape[0]
    assert n == 912673 and ne == 5308416
    mask = (xyz[:, 2] == 0.0).astype(np.uint8)
    theta = np.random.default_rng(9).standard_normal(ne)
    S = np.random.default_rng(10).choice(n, n // 100, replace=False)
    theta_obs = np.random.default_rng(11).standard_normal(ne)
    f = np.random.default_rng(5).uniform(-1.0, 1.0, n)
    s_obs, u_obs, _ = forward(xyz, conn, theta_obs, mask, f, 1, 1e-12)
    s_obs.close()
    s, u, b = forward(xyz, conn, theta, mask, f, 0, 1e-10)
    r = np.zeros(n)
    r[S] = u[S] - u_obs[S]
    g, st = s.adjoint_grad(r, u)
    assert st["status"] == 0 and st["relres"] <= 1e-10
    s.close()
    return dict(xyz=xyz, conn=conn, theta=theta, mask=mask, f=f, b=b, S=S, u_obs=u_obs, g=g)


def test_mixed_gradient_against_fp64_gradient(problem):
    p = problem
    s, u, _ = forward(p["xyz"], p["conn"], p["theta"], p["mask"], p["f"], 1, 1e-12)
    r = np.zeros(u.shape[0])
    r[p["S"]] = u[p["S"]] - p["u_obs"][p["S"]]
    gr, st = s.adjoint_grad(r, u)
    s.close()
    assert st["status"] == 0
    rel = np.linalg.norm(p["g"] - gr) / np.linalg.norm(gr)
    assert rel <= 1e-6, rel


def test_mixed_gradient_against_central_differences(problem):
    p = problem
    elems = np.random.default_rng(12).choice(p["conn"].shape[0], 32, replace=False)
    fd = gradcheck.central_differences(p["xyz"], p["conn"], p["theta"], p["mask"], p["b"], p["S"], p["u_obs"],
                                       elems, h=1e-6)
    rel = np.linalg.norm(fd - p["g"][elems]) / np.linalg.norm(fd)
    assert rel <= 1e-6, rel
