"""Parity with the oracle at the sizes of the workload's own configurations (needs a GB300):
the 2D 64^2 jittered-triangle Poisson problem and the 3D 64^3 Kuhn problem with
kappa = exp(g).  Pattern, assembled values, every level of the hierarchy and one V-cycle
are compared bit for bit; the PCG solution against a direct FP64 solve."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spl

import femgpu
import oracle as O
from femgpu import meshes
from test_oracle_pins import scaled_assembly_error

pytestmark = pytest.mark.gpu


def both(xyz, conn, kappa, f, mask, seed=1):
    rp, ci = O.build_pattern(xyz.shape[0], conn)
    v = O.assemble(xyz, conn, rp, ci, coef=kappa, lambda_mass=0.0)
    b = O.load_vector(xyz, conn, f)
    v, b = O.apply_dirichlet(rp, ci, v, mask, b)
    gx, ga = meshes.adjacency_from_pattern(rp, ci)
    orc = O.OracleAMG(rp, ci, v, gx, ga, seed=seed)
    s = femgpu.Solver(solverType=1, tolerance=1e-8, maxIters=300, flexibleCG=1, seed=seed)
    s.set_mesh(xyz, conn)
    s.assemble(kappa, 0.0)
    gb = s.load_vector(f)
    s.set_dirichlet(mask)
    gb[mask.astype(bool)] = 0.0
    grp, gci, gv = s.matrix()
    assert np.array_equal(grp, rp) and np.array_equal(gci, ci) and np.array_equal(gv, v)
    assert np.array_equal(gb, b)
    s.setup()
    return orc, s, sp.csr_matrix((v, ci, rp)), b


def check_hierarchy_and_cycle(orc, s):
    assert s.num_levels == orc.num_levels >= 2
    for l in range(orc.num_levels):
        go, oo = s.level(l), orc.level(l)
        for k in ("n", "nnz", "n_agg", "n_part", "nnz_p"):
            assert go[k] == oo[k], (l, k)
        for k in ("A_rowptr", "A_cols", "A_vals"):
            assert np.array_equal(go[k], oo[k]), (l, k)
        if oo["n_agg"]:
            for k in ("perm", "agg_idx", "part_idx", "P_rowptr", "P_cols", "P_vals"):
                assert np.array_equal(go[k], oo[k]), (l, k)
    r = np.random.default_rng(0).standard_normal(s.n)
    assert np.array_equal(s.vcycle(r), orc.vcycle(r))


def test_config_2d_64_jittered_triangles():
    xyz, tri, kappa, f, mask = meshes.poisson2d_problem(64, seed=1)
    assert xyz.shape[0] == 4225 and tri.shape[0] == 8192
    orc, s, A, b = both(xyz, tri, kappa, f, mask)
    assert A.nnz == 29057
    check_hierarchy_and_cycle(orc, s)
    x, st = s.solve(b)
    assert st["status"] == 0 and st["relres"] <= 1e-8
    xs = spl.spsolve(A.tocsc(), b)
    assert np.linalg.norm(x - xs) / np.linalg.norm(xs) < 1e-8
    xo, sto = orc.pcg(b, tol=1e-8, max_iters=300, flexible=True)
    assert abs(st["iterations"] - sto["iters"]) <= 1
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-8


def test_config_3d_64_kuhn():
    xyz, conn, kappa, f, mask = meshes.poisson3d_problem(64, sigma=1.0)
    assert xyz.shape[0] == 274625 and conn.shape[0] == 1572864
    orc, s, A, b = both(xyz, conn, kappa, f, mask)
    assert A.nnz == 4018753
    # the assembled values against the reference's cofactor-inverse element formula
    rp, ci = A.indptr, A.indices
    v_ref = O.assemble(xyz, conn, rp, ci, coef=kappa, lambda_mass=0.0, reference_formula=True)
    v_ref, _ = O.apply_dirichlet(rp, ci, v_ref, mask, None)
    assert scaled_assembly_error(rp, ci, A.data, v_ref) <= 1e-13
    check_hierarchy_and_cycle(orc, s)
    x, st = s.solve(b)
    assert st["status"] == 0 and st["relres"] <= 1e-8
    assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) <= 1.05e-8
    xo, sto = orc.pcg(b, tol=1e-8, max_iters=300, flexible=True)
    assert abs(st["iterations"] - sto["iters"]) <= 1
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-8
