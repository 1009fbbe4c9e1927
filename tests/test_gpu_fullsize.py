"""Size-independent properties at the 128^3 headline size (2,146,689 DOF, 31.8 M nnz),
where the CPU oracle is too slow to run inside a test (needs a GB300).

* the assembled operator is exactly symmetric (element matrices are symmetric and every
  entry sums the same element contributions in the same order);
* the mixed-precision PCG reaches the tolerance in the true FP64 residual;
* a V-cycle is deterministic and exactly homogeneous under scaling by 2: every operation
  on the way (rounding to FP32, products, sums, the relaxation, the FP64 coarse solve) is
  linear with fixed coefficients, and scaling by a power of two commutes with rounding."""
import numpy as np
import pytest
import scipy.sparse as sp

import femgpu
from femgpu import meshes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def headline():
    xyz, conn, kappa, f, mask = meshes.poisson3d_problem(128, sigma=2.0, kappa_seed=4, f_seed=5)
    s = femgpu.Solver(solverType=1, tolerance=1e-8, maxIters=300, flexibleCG=1, seed=1)
    s.set_mesh(xyz, conn)
    s.assemble(kappa, 0.0)
    s.set_dirichlet(mask)
    b = np.where(mask.astype(bool), 0.0, s.load_vector(f))
    rp, ci, v = s.matrix()
    s.setup()
    return s, sp.csr_matrix((v, ci, rp), shape=(rp.shape[0] - 1, rp.shape[0] - 1)), b


def test_operator_size_and_symmetry(headline):
    s, A, b = headline
    assert A.shape[0] == 2146689 and A.nnz == 31802497
    D = (A - A.T).tocsr()
    D.eliminate_zeros()
    assert D.nnz == 0


def test_solve_reaches_tolerance_in_the_true_residual(headline):
    s, A, b = headline
    x, st = s.solve(b)
    assert st["status"] == 0 and st["relres"] <= 1e-8
    assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) <= 1.05e-8


def test_vcycle_deterministic_and_exactly_homogeneous(headline):
    s, A, b = headline
    r = np.random.default_rng(0).standard_normal(A.shape[0])
    z1 = s.vcycle(r)
    assert np.array_equal(z1, s.vcycle(r))
    assert np.array_equal(s.vcycle(2.0 * r), 2.0 * z1)
    assert np.all(np.isfinite(z1)) and np.linalg.norm(z1) > 0
