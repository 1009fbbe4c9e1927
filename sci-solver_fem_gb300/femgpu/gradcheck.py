"""Central finite differences of a least-squares loss of the FEM solution with respect to
per-element log-coefficients, for checking femgpu_adjoint_grad.

The loss is L(theta) = 0.5 ||u(theta)[S] - u_obs[S]||^2 with A(theta) u = b, A(theta) =
sum_e exp(theta_e) K_e + Dirichlet elimination (what femgpu_assemble + femgpu_set_dirichlet
build).  For an element e and step h the central difference quotient

    (L(theta + h 1_e) - L(theta - h 1_e)) / (2 h)

is evaluated from two solves with the perturbed operators A+ = A(theta + h 1_e) and
A- = A(theta - h 1_e), both set up and solved by this library:

    u-  = A-^{-1} b,
    du  = u+ - u- = -A+^{-1} (A+ - A-) u-,      (A+ - A-) = 2 sinh(h) exp(theta_e) K_e,
    L+ - L- = 0.5 sum_S du (u+ + u- - 2 u_obs).

This is the same quotient as two independent loss evaluations, but the difference
u+ - u- is formed without cancellation: with h = 1e-6 a subtraction of two separately
solved u would lose about six of the sixteen digits, which is as large as the
agreement being tested.
"""
from __future__ import annotations

import numpy as np

from .capi import Solver


def element_stiffness(xyz, nodes):
    """Unit-coefficient P1 stiffness of one element (k x k): measure times the Gram
    matrix of the basis gradients."""
    k = len(nodes)
    dim = 3 if k == 4 else 2
    P = np.asarray(xyz, dtype=np.float64)[np.asarray(nodes)][:, :dim]
    M = np.concatenate([P, np.ones((k, 1))], axis=1)
    G = np.linalg.inv(M)[:dim, :].T  # k x dim: gradient of basis function a in row a
    meas = abs(np.linalg.det(M)) / (6.0 if dim == 3 else 2.0)
    return meas * (G @ G.T)


class _GpuSolves:
    """A(theta) u = rhs on the GPU: assemble, Dirichlet elimination, setup, PCG to tol."""

    def __init__(self, xyz, conn, mask, tol, precision):
        self.mask = mask
        self.s = Solver(solverType=1, tolerance=tol, maxIters=5000, flexibleCG=1, seed=1, precision=precision)
        self.s.set_mesh(xyz, conn)

    def __call__(self, theta, rhs):
        self.s.assemble(np.exp(theta), 0.0)
        self.s.set_dirichlet(self.mask)
        self.s.setup()
        u, _ = self.s.solve(rhs)
        return u

    def close(self):
        self.s.close()


def central_differences(xyz, conn, theta, mask, b, S, u_obs, elems, h=1e-6, tol=1e-12, precision=1, solve=None):
    """Central difference quotients of the loss for each element in `elems` (see the module
    docstring).  `solve(theta, rhs)` returns A(theta)^{-1} rhs; by default every solve runs on
    the GPU with the given precision setting to `tol`."""
    xyz = np.asarray(xyz, dtype=np.float64)
    conn = np.asarray(conn, dtype=np.int32)
    fixed = np.asarray(mask).astype(bool)
    bb = np.where(fixed, 0.0, b)
    own = solve is None
    if own:
        solve = _GpuSolves(xyz, conn, mask, tol, precision)
    out = np.zeros(len(elems))
    try:
        for q, e in enumerate(elems):
            tm = np.array(theta, dtype=np.float64)
            tp = tm.copy()
            tm[e] -= h
            tp[e] += h
            um = solve(tm, bb)
            nodes = conn[e]
            dA_u = 2.0 * np.sinh(h) * np.exp(theta[e]) * (element_stiffness(xyz, nodes) @ um[nodes])
            r = np.zeros_like(um)
            np.add.at(r, nodes, -dA_u)
            r[fixed] = 0.0
            du = solve(tp, r)
            up = um + du
            out[q] = 0.5 * float(np.dot(du[S], up[S] + um[S] - 2.0 * u_obs[S])) / (2.0 * h)
    finally:
        if own:
            solve.close()
    return out
