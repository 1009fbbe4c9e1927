"""Parity of the batched configurations with the CPU oracle (needs a GB300).

(a) the 64^3 Kuhn mesh (kappa = exp(g), seeds 4/5) with 64 seeded right-hand sides solved
    with one hierarchy: four of the columns against the oracle's PCG on the same column;
(b) the smallest (12^3) and the largest (40^3) cube of the 48-mesh batch (sizes from seed 7,
    coefficient seed 8 + i, load seed 1000 + i), solved together through femgpu_solve_batch:
    every level of each hierarchy bit for bit against the oracle's, and each solution
    against the oracle's PCG."""
import numpy as np
import pytest

import femgpu
import oracle as O
from femgpu import meshes

pytestmark = pytest.mark.gpu


def oracle_for(xyz, conn, kappa, mask, seed=1):
    rp, ci = O.build_pattern(xyz.shape[0], conn)
    v = O.assemble(xyz, conn, rp, ci, coef=kappa, lambda_mass=0.0)
    v, _ = O.apply_dirichlet(rp, ci, v, mask, None)
    gx, ga = meshes.adjacency_from_pattern(rp, ci)
    return O.OracleAMG(rp, ci, v, gx, ga, seed=seed), (rp, ci, v)


def test_multi_rhs_columns_against_oracle():
    xyz, conn, kappa, f, mask = meshes.poisson3d_problem(64, sigma=1.0, kappa_seed=4, f_seed=5)
    n = xyz.shape[0]
    s = femgpu.Solver(solverType=1, tolerance=1e-8, maxIters=500, flexibleCG=1, seed=1)
    s.set_mesh(xyz, conn)
    s.assemble(kappa, 0.0)
    s.set_dirichlet(mask)
    rng = np.random.default_rng(6)
    k = 64
    B = np.stack([np.where(mask.astype(bool), 0.0, s.load_vector(rng.uniform(-1.0, 1.0, n))) for _ in range(k)],
                 axis=1)
    s.setup()
    X, st = s.solve_multi(B)
    assert st["status"] == 0 and st["relres"] <= 1e-8
    orc, (rp, ci, v) = oracle_for(xyz, conn, kappa, mask)
    grp, gci, gv = s.matrix()
    assert np.array_equal(grp, rp) and np.array_equal(gci, ci) and np.array_equal(gv, v)
    for j in (0, 21, 42, 63):
        xo, sto = orc.pcg(B[:, j], tol=1e-8, max_iters=500, flexible=True)
        assert sto["status"] == 0
        assert np.linalg.norm(X[:, j] - xo) / np.linalg.norm(xo) <= 1e-8, j


def batch_problem(i, m):
    xyz, conn, kappa, f, mask = meshes.poisson3d_problem(m, sigma=1.0, kappa_seed=8 + i, f_seed=1000 + i)
    s = femgpu.Solver(solverType=1, tolerance=1e-8, maxIters=500, flexibleCG=1, seed=1)
    s.set_mesh(xyz, conn)
    s.assemble(kappa, 0.0)
    s.set_dirichlet(mask)
    b = np.where(mask.astype(bool), 0.0, s.load_vector(f))
    return s, b, (xyz, conn, kappa, mask)


def test_batch_extreme_meshes_against_oracle():
    sizes = np.random.default_rng(7).integers(12, 41, size=48)
    picks = [int(np.argmin(sizes)), int(np.argmax(sizes))]
    assert [int(sizes[i]) for i in picks] == [12, 40]
    probs = [batch_problem(i, int(sizes[i])) for i in picks]
    xs, stats, status = femgpu.solve_batch([p[0] for p in probs], [p[1] for p in probs])
    assert status == 0
    for (s, b, (xyz, conn, kappa, mask)), x, st in zip(probs, xs, stats):
        orc, _ = oracle_for(xyz, conn, kappa, mask)
        assert s.num_levels == orc.num_levels >= 2
        for l in range(orc.num_levels):
            go, oo = s.level(l), orc.level(l)
            for key in ("n", "nnz", "n_agg", "n_part", "nnz_p"):
                assert go[key] == oo[key], (l, key)
            for key in ("A_rowptr", "A_cols", "A_vals"):
                assert np.array_equal(go[key], oo[key]), (l, key)
            if oo["n_agg"]:
                for key in ("perm", "agg_idx", "part_idx", "P_rowptr", "P_cols", "P_vals"):
                    assert np.array_equal(go[key], oo[key]), (l, key)
        xo, sto = orc.pcg(b, tol=1e-8, max_iters=500, flexible=True)
        assert sto["status"] == 0 and abs(st["iterations"] - sto["iters"]) <= 1
        assert np.linalg.norm(x - xo) / np.linalg.norm(xo) <= 1e-8
