"""Pins the CPU oracle against the reference's own fixtures and libc (no GPU)."""
import ctypes
import os

import numpy as np
import pytest
import scipy.sparse as sp

import matio
import oracle as O
from femgpu import meshes


def test_glibc_rand_matches_libc():
    # randomizedMIS_GPU.cu:195-201 seeds the MIS with rand() after srand()
    libc = ctypes.CDLL("libc.so.6")
    for seed in (0, 1, 7, 12345, 2**31 - 1):
        libc.srand(seed)
        ref = np.array([libc.rand() for _ in range(2000)], np.int32)
        assert np.array_equal(O.glibc_rand(seed, 2000), ref)


def test_tet_mass_integrand_is_exact_p1_mass():
    # FEM3D quadrature: the collapsed 4^3 Gauss-Jacobi rule integrates P1 x P1 exactly;
    # with the reference's |0.125 det| Jacobian the table is 8x the unit-tet mass.
    m = O.tet_mass_integrand()
    diag = [0, 4, 7, 9]
    off = [1, 2, 3, 5, 6, 8]
    np.testing.assert_allclose(m[diag], 8 / 60, rtol=1e-12)
    np.testing.assert_allclose(m[off], 8 / 120, rtol=1e-12)


def test_tri_quadrature_weights():
    zx, wx, zy, wy = O.tri_quadrature()
    # the reference's Newton iteration stops at |step| < 1e-6, so zeros (and weights)
    # carry ~1e-12 errors
    assert abs(wx.sum() - 2.0) < 1e-10  # Gauss-Lobatto on [-1, 1]
    assert abs(wy.sum() - 2.0) < 1e-10  # Gauss-Radau(1,0) weights integrate (1 - y)
    assert zx[0] == -1 and zx[-1] == 1 and zy[0] == -1


def test_pattern_counts_kuhn():
    for n, nnz in ((2, None), (4, None)):
        xyz, conn = meshes.kuhn_cube(n)
        rp, ci = O.build_pattern(xyz.shape[0], conn)
        A = sp.csr_matrix((np.ones_like(ci, dtype=float), ci, rp))
        assert (A != A.T).nnz == 0
        rl = np.diff(rp)
        assert rl.max() == 15  # 14 Kuhn neighbours + diagonal
    # 64^3 count from the survey's brute-force check, scaled down: interior rows have 15
    xyz, conn = meshes.kuhn_cube(8)
    rp, ci = O.build_pattern(xyz.shape[0], conn)
    interior = np.array([(i // 81) in range(1, 8) and ((i // 9) % 9) in range(1, 8) and (i % 9) in range(1, 8)
                         for i in range(729)])
    assert np.all(np.diff(rp)[interior] == 15)


def test_assembly_properties():
    xyz, conn = meshes.kuhn_cube(4)
    rp, ci = O.build_pattern(xyz.shape[0], conn)
    K = sp.csr_matrix((O.assemble(xyz, conn, rp, ci, coef=np.ones(len(conn)), lambda_mass=0.0), ci, rp))
    A = sp.csr_matrix((O.assemble(xyz, conn, rp, ci), ci, rp))
    assert abs(K.sum(axis=1)).max() < 1e-13  # stiffness kills constants
    assert abs((A - K).sum() - 1.0) < 1e-12  # mass integrates to the volume
    x = xyz[:, 0]
    assert abs(x @ (K @ x) - 1.0) < 1e-12  # |grad x|^2 over the unit cube


def test_reference_fixture_simple_diagonal(ref_data):
    # sanity3D.cc: A = 79.9568 I, x = b / a
    A = matio.read(os.path.join(ref_data, "simple.mat"))
    b = matio.read(os.path.join(ref_data, "simpleb.mat"))
    ans = matio.read(os.path.join(ref_data, "simpleAns.mat"))
    assert A.shape == (5000, 5000) and A.nnz == 5000
    assert np.linalg.norm(A @ ans - b) / np.linalg.norm(b) < 1e-6


def test_oracle_solves_tetvol_known_answer(ref_data):
    # tetVol.cc: the SCIRun Laplacian fixture.  The stored answer satisfies
    # ||A ans - b|| / ||b|| ~ 6.7e-6; the oracle's AMG-PCG reaches 1e-8 and lands
    # within the reference test's bound ||x - ans|| < 25 by orders of magnitude.
    A = matio.read(os.path.join(ref_data, "tetVolA.mat"))
    b = matio.read(os.path.join(ref_data, "tetVolb.mat"))
    ans = matio.read(os.path.join(ref_data, "tetVolAns.mat"))
    rp, ci, v = A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data.copy()
    gx, ga = meshes.adjacency_from_pattern(rp, ci)
    amg = O.OracleAMG(rp, ci, v, gx, ga, seed=3)
    x, st = amg.pcg(b, tol=1e-8, max_iters=400, flexible=True)
    assert st["status"] == 0, st
    assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) <= 1.01e-8
    assert np.linalg.norm(x - ans) < 25.0
    assert np.linalg.norm(x - ans) / np.linalg.norm(ans) < 1e-4


def test_oracle_pcg_matches_direct_solve():
    xyz, conn, kappa, f, mask = meshes.poisson3d_problem(12)
    rp, ci = O.build_pattern(xyz.shape[0], conn)
    v = O.assemble(xyz, conn, rp, ci, coef=kappa, lambda_mass=0.0)
    b = O.load_vector(xyz, conn, f)
    v, b = O.apply_dirichlet(rp, ci, v, mask, b)
    A = sp.csr_matrix((v, ci, rp))
    xs = sp.linalg.spsolve(A.tocsc(), b)
    gx, ga = meshes.adjacency_from_pattern(rp, ci)
    for prec in (0, 1):
        amg = O.OracleAMG(rp, ci, v, gx, ga, seed=5, fp64_hierarchy=prec)
        x, st = amg.pcg(b, tol=1e-12, max_iters=200, flexible=True)
        assert st["status"] == 0
        assert np.linalg.norm(x - xs) / np.linalg.norm(xs) < 1e-9


def test_oracle_aggregation_invariants():
    xyz, conn = meshes.kuhn_cube(10)
    rp, ci = O.build_pattern(xyz.shape[0], conn)
    gx, ga = meshes.adjacency_from_pattern(rp, ci)
    o = O.oldmis(gx, ga, 90102, 512, seed=11)
    n = xyz.shape[0]
    assert sorted(o["perm"]) == list(range(n))
    assert np.array_equal(o["perm"][o["iperm"]], np.arange(n))
    sizes = np.diff(o["agg_idx"])
    assert sizes.min() >= 9  # runts (< 9) are removed and re-absorbed
    rows = np.diff(o["agg_idx"][o["part_idx"]])
    assert rows.max() <= 512
    # deterministic for a seed, different across seeds
    o2 = O.oldmis(gx, ga, 90102, 512, seed=11)
    assert np.array_equal(o["perm"], o2["perm"])
    o3 = O.oldmis(gx, ga, 90102, 512, seed=12)
    assert not np.array_equal(o["perm"], o3["perm"])


def test_oracle_operator_symmetric_and_vcycle_homogeneous():
    # the properties the full-size GPU test checks, on the oracle at a small size:
    # the assembled operator (Dirichlet rows and columns eliminated) is exactly
    # symmetric, and a V-cycle scales exactly with a power-of-two factor
    xyz, conn, kappa, f, mask = meshes.poisson3d_problem(8, sigma=2.0)
    rp, ci = O.build_pattern(xyz.shape[0], conn)
    v = O.assemble(xyz, conn, rp, ci, coef=kappa, lambda_mass=0.0)
    v, _ = O.apply_dirichlet(rp, ci, v, mask, None)
    A = sp.csr_matrix((v, ci, rp))
    D = (A - A.T).tocsr()
    D.eliminate_zeros()
    assert D.nnz == 0
    gx, ga = meshes.adjacency_from_pattern(rp, ci)
    for prec in (0, 1):
        amg = O.OracleAMG(rp, ci, v, gx, ga, seed=2, fp64_hierarchy=prec)
        r = np.random.default_rng(1).standard_normal(xyz.shape[0])
        z = amg.vcycle(r)
        assert np.array_equal(amg.vcycle(2.0 * r), 2.0 * z)
        assert np.array_equal(amg.vcycle(0.25 * r), 0.25 * z)


def scaled_assembly_error(rp, ci, v_lib, v_ref):
    """max |a_lib - a_ref| / sqrt(|a_ii a_jj|) over the pattern (entries scaled by their
    diagonal pair, so structurally near-zero couplings are measured against the row scale)."""
    n = rp.shape[0] - 1
    rows = np.repeat(np.arange(n), np.diff(rp))
    diag = np.zeros(n)
    on = ci == rows
    diag[rows[on]] = np.abs(v_ref[on])
    scale = np.sqrt(diag[rows] * diag[ci])
    return float(np.max(np.abs(v_lib - v_ref) / scale))


@pytest.mark.parametrize("case", ["poisson_32_kappa", "poisson_16_sigma2", "kuhn_mass"])
def test_library_element_formula_matches_reference_formula(case):
    # on Kuhn cubes of 2^k cells per edge (the configurations' meshes: exact coordinates)
    # the fused multiply-add gradients (what the GPU assembles) agree with the reference's
    # 4x4 cofactor inverse to 1e-13 relative to the row scale
    rng = np.random.default_rng(5)
    if case == "poisson_32_kappa":
        xyz, conn, kappa, f, mask = meshes.poisson3d_problem(32, sigma=1.0)
        kw = dict(coef=kappa, lambda_mass=0.0)
    elif case == "poisson_16_sigma2":
        xyz, conn, kappa, f, mask = meshes.poisson3d_problem(16, sigma=2.0, kappa_seed=4)
        kw = dict(coef=kappa, lambda_mass=0.0)
    else:
        xyz, conn = meshes.kuhn_cube(8)
        kw = dict(coef=np.exp(rng.standard_normal(conn.shape[0])), lambda_mass=2.5)
    rp, ci = O.build_pattern(xyz.shape[0], conn)
    v_lib = O.assemble(xyz, conn, rp, ci, **kw)
    v_ref = O.assemble(xyz, conn, rp, ci, reference_formula=True, **kw)
    assert scaled_assembly_error(rp, ci, v_lib, v_ref) <= 1e-13


def exact_stiffness(p):
    """Unit-coefficient P1 stiffness of one tetrahedron in exact rational arithmetic."""
    from fractions import Fraction
    P = [[Fraction(float(v)) for v in row] for row in p]
    a, b, c = ([P[q][d] - P[0][d] for d in range(3)] for q in (1, 2, 3))

    def cross(u, v):
        return [u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]]

    bc, ca, ab = cross(b, c), cross(c, a), cross(a, b)
    det = sum(a[d] * bc[d] for d in range(3))
    g = [None, [t / det for t in bc], [t / det for t in ca], [t / det for t in ab]]
    g[0] = [-(g[1][d] + g[2][d] + g[3][d]) for d in range(3)]
    vol = abs(det) / 6
    return np.array([[float(vol * sum(g[i][d] * g[j][d] for d in range(3))) for j in range(4)] for i in range(4)])


@pytest.mark.parametrize("mesh", ["tetVol", "CubeMesh_size256step16_correct", "jittered", "kuhn9"])
def test_element_formulas_against_exact_arithmetic(ref_data, mesh):
    # Where coordinates are not short binary fractions (the reference's own meshes, a
    # jittered cube, a cube of 9 cells per edge) the two formulas differ by up to a few
    # 1e-12: the reference's cofactor inverse of [x y z 1] loses digits there, while the
    # edge-vector gradients stay within a few units in the last place of the exact element
    # matrix.
    import femgpu
    if mesh == "jittered":
        xyz, conn = meshes.kuhn_cube(9)
        xyz = xyz + np.random.default_rng(5).uniform(-0.03, 0.03, xyz.shape)
    elif mesh == "kuhn9":
        xyz, conn = meshes.kuhn_cube(9)
    else:
        xyz, conn, lab = femgpu.read_tetgen(os.path.join(ref_data, mesh))
    worst_lib = worst_ref = 0.0
    for e in np.random.default_rng(0).choice(conn.shape[0], 60, replace=False):
        c = conn[e]
        loc = np.arange(4, dtype=np.int32).reshape(1, 4)
        rp, ci = O.build_pattern(4, loc)
        Ke = exact_stiffness(xyz[c])
        scale = np.sqrt(np.outer(np.abs(np.diag(Ke)), np.abs(np.diag(Ke))))
        for ref, name in ((False, "lib"), (True, "ref")):
            v = O.assemble(xyz[c], loc, rp, ci, coef=np.ones(1), lambda_mass=0.0, reference_formula=ref)
            K = sp.csr_matrix((v, ci, rp)).toarray()
            err = float(np.max(np.abs(K - Ke) / scale))
            if name == "lib":
                worst_lib = max(worst_lib, err)
            else:
                worst_ref = max(worst_ref, err)
    assert worst_lib <= 2e-15, worst_lib
    assert worst_ref >= worst_lib
