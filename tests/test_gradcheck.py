"""The central-difference evaluation used to check the adjoint gradient (CPU, scipy solves):
it equals the plain difference of two loss evaluations at a step where cancellation is
harmless, and agrees with the FP64 adjoint gradient at h = 1e-6."""
import numpy as np

import adjoint_ref as R
from femgpu import gradcheck


def scipy_solve(xyz, conn, mask):
    return lambda theta, rhs: R.solve(xyz, conn, theta, mask, rhs)


def test_difference_form_equals_two_loss_evaluations():
    xyz, conn, theta, mask, b, S, u_obs = R.problem(5, dim=3)
    elems = [0, 17, 301]
    h = 1e-2
    fd = gradcheck.central_differences(xyz, conn, theta, mask, b, S, u_obs, elems, h=h,
                                       solve=scipy_solve(xyz, conn, mask))
    for q, e in enumerate(elems):
        tp, tm = theta.copy(), theta.copy()
        tp[e] += h
        tm[e] -= h
        Lp, _ = R.loss_and_dLdu(R.solve(xyz, conn, tp, mask, b), S, u_obs)
        Lm, _ = R.loss_and_dLdu(R.solve(xyz, conn, tm, mask, b), S, u_obs)
        assert abs(fd[q] - (Lp - Lm) / (2 * h)) <= 1e-9 * abs(fd[q])


def test_central_differences_match_the_adjoint_gradient():
    for dim, n in ((3, 6), (2, 12)):
        xyz, conn, theta, mask, b, S, u_obs = R.problem(n, dim=dim)
        u = R.solve(xyz, conn, theta, mask, b)
        _, dLdu = R.loss_and_dLdu(u, S, u_obs)
        g = R.gradient(xyz, conn, theta, mask, dLdu, u)
        elems = np.random.default_rng(12).choice(conn.shape[0], 16, replace=False)
        fd = gradcheck.central_differences(xyz, conn, theta, mask, b, S, u_obs, elems, h=1e-6,
                                           solve=scipy_solve(xyz, conn, mask))
        assert np.linalg.norm(fd - g[elems]) / np.linalg.norm(g[elems]) <= 1e-8


def test_element_stiffness_matches_basis_gradients():
    xyz, conn, theta, mask, b, S, u_obs = R.problem(4, dim=3)
    meas, G = R.basis_gradients(xyz, conn)
    for e in (0, 5, 99):
        K = gradcheck.element_stiffness(xyz, conn[e])
        assert np.allclose(K, meas[e] * G[e] @ G[e].T, rtol=1e-13, atol=1e-15)
        assert np.allclose(K.sum(axis=1), 0.0, atol=1e-14)
