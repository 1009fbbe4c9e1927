"""FP64 reference for the log-coefficient gradient (test infrastructure).

The operator comes from the CPU oracle's assembly (A = sum_e exp(theta_e) K_e with the
Dirichlet rows eliminated), solves are scipy direct solves, and the element gradient
is restated with numpy: dL/dtheta_e = -exp(theta_e) * lambda_e^T K_e u_e, K_e the
unit-coefficient P1 stiffness (volume times the Gram matrix of the basis gradients).
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spl

import oracle as O


def operator(xyz, conn, theta, mask):
    rp, ci = O.build_pattern(xyz.shape[0], conn)
    v = O.assemble(xyz, conn, rp, ci, coef=np.exp(theta), lambda_mass=0.0)
    v, _ = O.apply_dirichlet(rp, ci, v, mask, None)
    return sp.csr_matrix((v, ci, rp), shape=(xyz.shape[0], xyz.shape[0])).tocsc()


def solve(xyz, conn, theta, mask, b):
    A = operator(xyz, conn, theta, mask)
    return spl.spsolve(A, np.where(mask.astype(bool), 0.0, b))


def basis_gradients(xyz, conn):
    """Per element: (measure, gradients of the P1 basis functions, shape (ne, k, dim))."""
    k = conn.shape[1]
    dim = 3 if k == 4 else 2
    P = xyz[conn][:, :, :dim]                      # ne x k x dim
    M = np.concatenate([P, np.ones(P.shape[:2] + (1,))], axis=2)  # rows [x y (z) 1]
    Minv = np.linalg.inv(M)                         # columns = basis coefficients
    G = np.transpose(Minv[:, :dim, :], (0, 2, 1))   # ne x k x dim
    fact = 6.0 if dim == 3 else 2.0
    meas = np.abs(np.linalg.det(M)) / fact
    return meas, G


def gradient(xyz, conn, theta, mask, dLdu, u):
    """Adjoint gradient dL/dtheta for the loss with derivative dLdu at the solution u."""
    A = operator(xyz, conn, theta, mask)
    lam = spl.spsolve(A, np.where(mask.astype(bool), 0.0, dLdu))
    meas, G = basis_gradients(xyz, conn)
    gl = np.einsum("ek,ekd->ed", lam[conn], G)
    gu = np.einsum("ek,ekd->ed", u[conn], G)
    return -np.exp(theta) * meas * np.einsum("ed,ed->e", gl, gu)


def problem(n, dim=3, seed=9, frac=0.05):
    """Small version of the differentiation workload: theta ~ N(0,1), loss
    0.5 ||u[S] - u_obs||^2 over a random vertex subset S, u_obs from a second theta."""
    from femgpu import meshes
    if dim == 3:
        xyz, conn = meshes.kuhn_cube(n)
        mask = (xyz[:, 2] == 0.0).astype(np.uint8)
    else:
        xyz, conn = meshes.jittered_square(n)
        mask = ((xyz[:, 0] == 0) | (xyz[:, 0] == 1) | (xyz[:, 1] == 0) | (xyz[:, 1] == 1)).astype(np.uint8)
    rng = np.random.default_rng(seed)
    theta = rng.standard_normal(conn.shape[0])
    theta_obs = rng.standard_normal(conn.shape[0])
    f = rng.uniform(-1.0, 1.0, xyz.shape[0])
    b = O.load_vector(xyz, conn, f)
    S = rng.choice(xyz.shape[0], max(1, int(frac * xyz.shape[0])), replace=False)
    u_obs = solve(xyz, conn, theta_obs, mask, b)
    return xyz, conn, theta, mask, b, S, u_obs


def loss_and_dLdu(u, S, u_obs):
    r = np.zeros_like(u)
    r[S] = u[S] - u_obs[S]
    return 0.5 * float(np.sum(r[S] ** 2)), r
