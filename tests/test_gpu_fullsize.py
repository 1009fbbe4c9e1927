"""Parity at the 128^3 headline configuration (2,146,689 DOF, 31.8 M nnz, kappa = exp(2 g)),
needs a GB300.

The CPU oracle builds the same problem (its assembly, its hierarchy on every host core, a
few seconds on the GPU host), and the CUDA path is compared with it:
* the sparsity pattern, the assembled values and the load vector bit for bit, and the
  assembled values within 1e-13 (relative to the row scale) of the reference's own
  cofactor-inverse element formula;
* every level of the hierarchy bit for bit: A, the permutation, the aggregate and
  partition offsets and P;
* one V-cycle bit for bit;
* the PCG iteration count within one of the oracle's, and the solution within 1e-8 of an
  FP64-hierarchy PCG solved to 1e-12.
Size-independent properties of the same operator are checked as well: exact symmetry, the
solve's true FP64 residual, and a deterministic V-cycle that is exactly homogeneous under
scaling by 2 (every operation on the way is linear with fixed coefficients, and scaling by
a power of two commutes with rounding)."""
import numpy as np
import pytest
import scipy.sparse as sp

import femgpu
import oracle as O
from femgpu import meshes
from test_oracle_pins import scaled_assembly_error

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
    return dict(s=s, A=sp.csr_matrix((v, ci, rp), shape=(rp.shape[0] - 1, rp.shape[0] - 1)), b=b,
                problem=(xyz, conn, kappa, f, mask))


@pytest.fixture(scope="module")
def oracle_side(headline):
    xyz, conn, kappa, f, mask = headline["problem"]
    rp, ci = O.build_pattern(xyz.shape[0], conn)
    v = O.assemble(xyz, conn, rp, ci, coef=kappa, lambda_mass=0.0)
    b = O.load_vector(xyz, conn, f)
    v, b = O.apply_dirichlet(rp, ci, v, mask, b)
    gx, ga = meshes.adjacency_from_pattern(rp, ci)
    orc = O.OracleAMG(rp, ci, v, gx, ga, seed=1)
    return dict(orc=orc, rp=rp, ci=ci, v=v, b=b)


def test_operator_size_and_symmetry(headline):
    A = headline["A"]
    assert A.shape[0] == 2146689 and A.nnz == 31802497
    D = (A - A.T).tocsr()
    D.eliminate_zeros()
    assert D.nnz == 0


def test_pattern_values_and_load_vector_bit_exact(headline, oracle_side):
    A = headline["A"]
    assert np.array_equal(A.indptr, oracle_side["rp"]) and np.array_equal(A.indices, oracle_side["ci"])
    assert np.array_equal(A.data, oracle_side["v"])
    assert np.array_equal(headline["b"], oracle_side["b"])


def test_assembled_values_against_reference_element_formula(headline):
    # the reference's 4x4 cofactor inverse per element: within 1e-13 of the row scale
    xyz, conn, kappa, f, mask = headline["problem"]
    A = headline["A"]
    v_ref = O.assemble(xyz, conn, A.indptr, A.indices, coef=kappa, lambda_mass=0.0, reference_formula=True)
    v_ref, _ = O.apply_dirichlet(A.indptr, A.indices, v_ref, mask, None)
    assert scaled_assembly_error(A.indptr, A.indices, A.data, v_ref) <= 1e-13


def test_every_level_bit_exact(headline, oracle_side):
    s, orc = headline["s"], oracle_side["orc"]
    assert s.num_levels == orc.num_levels >= 3
    for l in range(orc.num_levels):
        go, oo = s.level(l), orc.level(l)
        for k in ("n", "nnz", "n_agg", "n_part", "nnz_p"):
            assert go[k] == oo[k], (l, k)
        for k in ("A_rowptr", "A_cols", "A_vals"):
            assert np.array_equal(go[k], oo[k]), (l, k)
        if oo["n_agg"]:
            for k in ("perm", "agg_idx", "part_idx", "P_rowptr", "P_cols", "P_vals"):
                assert np.array_equal(go[k], oo[k]), (l, k)


def test_vcycle_bit_exact(headline, oracle_side):
    r = np.random.default_rng(0).standard_normal(headline["A"].shape[0])
    assert np.array_equal(headline["s"].vcycle(r), oracle_side["orc"].vcycle(r))


def test_pcg_against_oracle_and_fp64_solve(headline, oracle_side):
    s, A, b = headline["s"], headline["A"], headline["b"]
    x, st = s.solve(b)
    assert st["status"] == 0 and st["relres"] <= 1e-8
    assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) <= 1.05e-8
    xo, sto = oracle_side["orc"].pcg(b, tol=1e-8, max_iters=300, flexible=True)
    assert sto["status"] == 0 and abs(st["iterations"] - sto["iters"]) <= 1
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) <= 1e-8
    ref = femgpu.Solver(solverType=1, tolerance=1e-12, maxIters=2000, flexibleCG=1, seed=1, precision=1)
    ref.set_matrix_csr(A.indptr, A.indices, A.data)
    x12, st12 = ref.solve(b)
    ref.close()
    assert st12["status"] == 0 and st12["relres"] <= 1e-12
    assert np.linalg.norm(x - x12) / np.linalg.norm(x12) <= 1e-8


def test_vcycle_deterministic_and_exactly_homogeneous(headline):
    s = headline["s"]
    r = np.random.default_rng(1).standard_normal(headline["A"].shape[0])
    z1 = s.vcycle(r)
    assert np.array_equal(z1, s.vcycle(r))
    assert np.array_equal(s.vcycle(2.0 * r), 2.0 * z1)
    assert np.all(np.isfinite(z1)) and np.linalg.norm(z1) > 0
