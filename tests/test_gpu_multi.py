"""Several right-hand sides with one hierarchy (needs a GB300)."""
import numpy as np
import pytest

import femgpu
from femgpu import meshes

pytestmark = pytest.mark.gpu


def multi_problem(n, precision=0, seed=6):
    xyz, conn, kappa, f, mask = meshes.poisson3d_problem(n, sigma=2.0)
    s = femgpu.Solver(solverType=1, tolerance=1e-8, maxIters=300, flexibleCG=1, seed=seed, precision=precision)
    s.set_mesh(xyz, conn)
    s.assemble(kappa, 0.0)
    s.set_dirichlet(mask)
    return s, xyz, mask


@pytest.mark.parametrize("precision,k", [(0, 8), (0, 11), (1, 5)])
def test_multi_rhs_matches_single_solves(precision, k):
    # the block solve runs every column's own PCG (eight in lockstep, block kernels);
    # each column agrees with the single-column solve of the same right-hand side
    s, xyz, mask = multi_problem(14, precision)
    rng = np.random.default_rng(6)
    B = np.stack([np.where(mask.astype(bool), 0.0, s.load_vector(rng.uniform(-1, 1, xyz.shape[0])))
                  for _ in range(k)], axis=1)
    s.setup()
    launches0 = femgpu.kernel_launches()
    X, st = s.solve_multi(B)
    assert femgpu.kernel_launches() > launches0
    assert st["status"] == 0 and st["relres"] <= 1e-8
    iters = 0
    for j in range(k):
        x, sj = s.solve(B[:, j])
        iters += sj["iterations"]
        assert np.linalg.norm(X[:, j] - x) / np.linalg.norm(x) <= 1e-8, j
    assert abs(st["iterations"] - iters) <= k


def test_multi_rhs_nonzero_initial_guess_and_zero_column():
    s, xyz, mask = multi_problem(10)
    rng = np.random.default_rng(2)
    n = xyz.shape[0]
    B = np.stack([np.where(mask.astype(bool), 0.0, s.load_vector(rng.uniform(-1, 1, n))) for _ in range(3)], axis=1)
    B[:, 1] = 0.0  # a zero right-hand side is solved by x = 0 at once
    X0 = np.where(mask.astype(bool)[:, None], 0.0, rng.standard_normal((n, 3)) * 0.1)
    X0[:, 1] = 0.0
    s.setup()
    X, st = s.solve_multi(B, X0)
    assert st["status"] == 0
    assert np.all(X[:, 1] == 0.0)
    rp, ci, v = s.matrix()
    import scipy.sparse as sp
    A = sp.csr_matrix((v, ci, rp))
    for j in (0, 2):
        assert np.linalg.norm(B[:, j] - A @ X[:, j]) / np.linalg.norm(B[:, j]) <= 1.05e-8


def test_multi_rhs_coarsest_only_dense_solve_on_tensor_cores():
    # 5^3 vertices is below topSize: the hierarchy is the coarsest level alone, so the
    # block preconditioner is the dense FP64 inverse applied by the DMMA kernel, and one
    # PCG iteration solves every column
    xyz, conn, kappa, f, mask = meshes.poisson3d_problem(4, sigma=1.0)
    s = femgpu.Solver(solverType=1, tolerance=1e-10, maxIters=50, flexibleCG=1, seed=1)
    s.set_mesh(xyz, conn)
    s.assemble(kappa, 0.0)
    s.set_dirichlet(mask)
    s.setup()
    assert s.num_levels == 1
    rng = np.random.default_rng(4)
    n = xyz.shape[0]
    B = np.where(mask.astype(bool)[:, None], 0.0, rng.uniform(-1, 1, (n, 9)))
    X, st = s.solve_multi(B)
    rp, ci, v = s.matrix()
    import scipy.sparse as sp
    A = sp.csr_matrix((v, ci, rp)).toarray()
    Xd = np.linalg.solve(A, B)
    assert np.linalg.norm(X - Xd) / np.linalg.norm(Xd) <= 1e-10
    assert st["status"] == 0 and st["iterations"] <= 2 * 9


def test_multi_rhs_rejects_bad_leading_dimension():
    xyz, conn = meshes.kuhn_cube(3)
    s = femgpu.Solver(solverType=1)
    s.set_mesh(xyz, conn)
    s.assemble()
    import ctypes as C
    from femgpu import capi
    st = capi.SolveStats()
    # ldb smaller than the row count is refused before any device access
    assert capi.lib().femgpu_solve_multi_device(s.h, 1, C.c_void_p(16), 1, C.c_void_p(16), 1, C.byref(st)) == 1


def test_in_place_solve_matches_copying_solve():
    xyz, conn, kappa, f, mask = meshes.poisson3d_problem(10, sigma=2.0)
    s = femgpu.Solver(solverType=1, tolerance=1e-8, maxIters=300, flexibleCG=1, seed=6)
    s.set_mesh(xyz, conn)
    s.assemble(kappa, 0.0)
    s.set_dirichlet(mask)
    b = np.where(mask.astype(bool), 0.0, s.load_vector(f))
    s.setup()
    x1, st1 = s.solve(b)
    out = np.zeros(s.n)
    x2, st2 = s.solve(b, out=out)
    assert x2 is out and np.array_equal(x1, out) and st1["iterations"] == st2["iterations"]
    with pytest.raises(ValueError):
        s.solve(b, out=np.zeros(s.n, dtype=np.float32))
