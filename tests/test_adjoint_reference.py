"""The FP64 reference gradient against central finite differences (CPU only)."""
import numpy as np
import pytest

import adjoint_ref as R


@pytest.mark.parametrize("dim,n", [(3, 5), (2, 12)])
def test_reference_gradient_matches_central_differences(dim, n):
    xyz, conn, theta, mask, b, S, u_obs = R.problem(n, dim=dim)
    u = R.solve(xyz, conn, theta, mask, b)
    L, dLdu = R.loss_and_dLdu(u, S, u_obs)
    g = R.gradient(xyz, conn, theta, mask, dLdu, u)
    rng = np.random.default_rng(12)
    h = 1e-6
    elems = rng.choice(conn.shape[0], 16, replace=False)
    fd = np.zeros(len(elems))
    for q, e in enumerate(elems):
        tp, tm = theta.copy(), theta.copy()
        tp[e] += h
        tm[e] -= h
        Lp, _ = R.loss_and_dLdu(R.solve(xyz, conn, tp, mask, b), S, u_obs)
        Lm, _ = R.loss_and_dLdu(R.solve(xyz, conn, tm, mask, b), S, u_obs)
        fd[q] = (Lp - Lm) / (2 * h)
    # central differences with h = 1e-6 against the adjoint formula, norm-wise
    rel = np.linalg.norm(fd - g[elems]) / np.linalg.norm(g[elems])
    assert rel <= 1e-6, rel
