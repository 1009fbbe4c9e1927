"""CUDA path vs the CPU oracle, through the C ABI (needs a GB300)."""
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spl

import matio
import oracle as O
import femgpu
from femgpu import meshes

pytestmark = pytest.mark.gpu


def oracle_operator(xyz, conn, coef=None, labels=None, lam=1.0, mask=None, f=None):
    rp, ci = O.build_pattern(xyz.shape[0], conn)
    v = O.assemble(xyz, conn, rp, ci, labels=labels, coef=coef, lambda_mass=lam)
    b = O.load_vector(xyz, conn, f) if f is not None else None
    if mask is not None:
        v, b = O.apply_dirichlet(rp, ci, v, mask, b)
    return rp, ci, v, b


def gpu_operator(xyz, conn, coef=None, labels=None, lam=1.0, mask=None, f=None, **opts):
    s = femgpu.Solver(**opts)
    s.set_mesh(xyz, conn, labels)
    s.assemble(coef, lam)
    b = s.load_vector(f) if f is not None else None
    if mask is not None:
        s.set_dirichlet(mask)
        b = np.where(mask.astype(bool), 0.0, b) if b is not None else None
    return s, b


@pytest.mark.parametrize("case", ["tet_reference", "tet_poisson", "tri_poisson"])
def test_pattern_and_assembly_bit_exact(case):
    rng = np.random.default_rng(3)
    if case == "tet_reference":
        xyz, conn = meshes.kuhn_cube(7)
        xyz = xyz + rng.uniform(-0.02, 0.02, xyz.shape)
        labels = rng.integers(0, 7, conn.shape[0]).astype(np.int32)
        kw = dict(labels=labels, lam=1.0)
    elif case == "tet_poisson":
        xyz, conn, kappa, f, mask = meshes.poisson3d_problem(9)
        kw = dict(coef=kappa, lam=0.0, mask=mask, f=f)
    else:
        xyz, conn, kappa, f, mask = meshes.poisson2d_problem(20)
        kw = dict(coef=kappa, lam=0.0, mask=mask, f=f)
    rp, ci, v, b = oracle_operator(xyz, conn, **kw)
    s, gb = gpu_operator(xyz, conn, **kw)
    grp, gci, gv = s.matrix()
    assert np.array_equal(grp, rp) and np.array_equal(gci, ci)
    assert np.array_equal(gv, v), np.abs(gv - v).max()
    if b is not None:
        assert np.array_equal(gb, b)


def test_reference_mesh_assembly_bit_exact(ref_data):
    xyz, conn, lab = femgpu.read_tetgen(os.path.join(ref_data, "tetVol"))
    rp, ci, v, _ = oracle_operator(xyz, conn, labels=lab, lam=1.0)
    s, _ = gpu_operator(xyz, conn, labels=lab, lam=1.0)
    grp, gci, gv = s.matrix()
    assert np.array_equal(grp, rp) and np.array_equal(gci, ci) and np.array_equal(gv, v)
    xyz, tri = femgpu.read_ply(os.path.join(ref_data, "simple.ply"))
    rp, ci, v, _ = oracle_operator(xyz, tri, lam=1.0)
    s, _ = gpu_operator(xyz, tri, lam=1.0)
    grp, gci, gv = s.matrix()
    assert np.array_equal(grp, rp) and np.array_equal(gci, ci) and np.array_equal(gv, v)


def build_both(n=14, seed=7, precision=0, sigma=1.0):
    xyz, conn, kappa, f, mask = meshes.poisson3d_problem(n, sigma=sigma)
    rp, ci, v, b = oracle_operator(xyz, conn, coef=kappa, lam=0.0, mask=mask, f=f)
    gx, ga = meshes.adjacency_from_pattern(rp, ci)
    orc = O.OracleAMG(rp, ci, v, gx, ga, seed=seed, fp64_hierarchy=precision)
    s, gb = gpu_operator(xyz, conn, coef=kappa, lam=0.0, mask=mask, f=f, seed=seed, precision=precision,
                         solverType=1, tolerance=1e-8, maxIters=300, flexibleCG=1)
    s.setup()
    return orc, s, (rp, ci, v, b)


@pytest.mark.parametrize("precision", [0, 1])
def test_hierarchy_matches_oracle(precision):
    orc, s, _ = build_both(n=16, seed=7, precision=precision)
    assert s.num_levels == orc.num_levels >= 2
    for l in range(orc.num_levels):
        go, oo = s.level(l), orc.level(l)
        for k in ("n", "nnz", "n_agg", "n_part", "nnz_p"):
            assert go[k] == oo[k], (l, k)
        assert np.array_equal(go["A_rowptr"], oo["A_rowptr"]) and np.array_equal(go["A_cols"], oo["A_cols"])
        assert np.array_equal(go["A_vals"], oo["A_vals"]), (l, np.abs(go["A_vals"] - oo["A_vals"]).max())
        if oo["n_agg"]:
            for k in ("perm", "agg_idx", "part_idx", "P_rowptr", "P_cols"):
                assert np.array_equal(go[k], oo[k]), (l, k)
            assert np.array_equal(go["P_vals"], oo["P_vals"]), (l, np.abs(go["P_vals"] - oo["P_vals"]).max())


def test_large_hierarchy_with_long_rap_rows():
    # 96^3 (912,673 DOF): level 2's Galerkin rows exceed the 8192-product shared-memory
    # sort and take the dense-accumulator path; values must still match bit for bit.
    orc, s, _ = build_both(n=96, seed=1, precision=0, sigma=2.0)
    assert s.num_levels == orc.num_levels >= 4
    for l in range(orc.num_levels):
        go, oo = s.level(l), orc.level(l)
        assert go["nnz"] == oo["nnz"] and go["n_agg"] == oo["n_agg"]
        if oo["n_agg"]:
            assert np.array_equal(go["perm"], oo["perm"]) and np.array_equal(go["agg_idx"], oo["agg_idx"])
        if l > 0:
            assert np.array_equal(go["A_cols"], oo["A_cols"]) and np.array_equal(go["A_vals"], oo["A_vals"])


@pytest.mark.parametrize("seed", [1, 2, 99])
def test_aggregates_bit_exact_across_seeds(seed):
    orc, s, _ = build_both(n=12, seed=seed)
    for l in range(orc.num_levels - 1):
        go, oo = s.level(l), orc.level(l)
        assert np.array_equal(go["perm"], oo["perm"])
        assert np.array_equal(go["agg_idx"], oo["agg_idx"])
        assert np.array_equal(go["part_idx"], oo["part_idx"])


@pytest.mark.parametrize("precision,n", [(0, 14), (1, 14), (0, 40), (1, 40)])
def test_vcycle_matches_oracle(precision, n):
    # n = 40: coarse levels run the shared-memory smoother on multi-CTA clusters
    orc, s, (rp, ci, v, b) = build_both(n=n, seed=5, precision=precision, sigma=2.0)
    r = np.random.default_rng(0).standard_normal(rp.shape[0] - 1)
    zg, zo = s.vcycle(r), orc.vcycle(r)
    assert np.array_equal(zg, zo), np.abs(zg - zo).max() / np.abs(zo).max()


@pytest.mark.parametrize("precision", [0, 1])
def test_pcg_solution_against_fp64_direct_solve(precision):
    orc, s, (rp, ci, v, b) = build_both(n=20, seed=3, precision=precision, sigma=2.0)
    A = sp.csr_matrix((v, ci, rp))
    x, st = s.solve(b)
    assert st["status"] == 0 and st["relres"] <= 1e-8
    true_rel = np.linalg.norm(b - A @ x) / np.linalg.norm(b)
    assert true_rel <= 1.05e-8
    xs = spl.spsolve(A.tocsc(), b)  # FP64 reference solution
    err = np.linalg.norm(x - xs) / np.linalg.norm(xs)
    assert err < 1e-8, err  # the oracle's own PCG reaches 1.7e-9 on this problem
    xo, sto = orc.pcg(b, tol=1e-8, max_iters=300, flexible=True)
    assert abs(st["iterations"] - sto["iters"]) <= 1
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-8


def test_single_vcycle_solver_type_0():
    orc, s, (rp, ci, v, b) = build_both(n=10, seed=4)
    s2 = femgpu.Solver(solverType=0, seed=4)
    s2.set_matrix_csr(rp, ci, v)
    x, st = s2.solve(b)
    assert st["iterations"] == 1
    # one V-cycle applied to b, as AMG_SOLVER does (amg.cu:150-160)
    gx, ga = meshes.adjacency_from_pattern(rp, ci)
    orc2 = O.OracleAMG(rp, ci, v, gx, ga, seed=4)
    assert np.array_equal(x, orc2.vcycle(b))


def reference_mat_override(rp, ci, A):
    """FEMSolver::readMatlabSparseMatrix (src/FEMSolver.cu:342-354): mesh-pattern entries
    set to 1e-12 and added to the file matrix (union of the two patterns)."""
    M = sp.csr_matrix((np.full(ci.shape[0], 1e-12), ci, rp), shape=A.shape)
    U = (A + M).tocsr()
    U.sort_indices()
    return U


@pytest.mark.parametrize("name,mesh,tol", [("tetVol", "tet", 25.0), ("simple", "tet", 1.0),
                                           ("simpleTri", "tri", 100.0)])
def test_reference_end_to_end_fixtures(ref_data, name, mesh, tol):
    # sanity3D.cc / tetVol.cc / sanity2D.cc through the drop-in flow: mesh -> assemble
    # -> MAT override -> solve; the reference's assertion plus a residual check.
    if mesh == "tet":
        base = "tetVol" if name == "tetVol" else "simple"
        xyz, conn, lab = femgpu.read_tetgen(os.path.join(ref_data, base))
        matA, matb, ans = f"{name}A.mat" if name == "tetVol" else "simple.mat", f"{name}b.mat", f"{name}Ans.mat"
    else:
        xyz, conn = femgpu.read_ply(os.path.join(ref_data, "simple.ply"))
        lab = None
        matA, matb, ans = "simpleTri.mat", "simpleTrib.mat", "simpleTriAns.mat"
    s = femgpu.Solver(solverType=1, tolerance=1e-8, maxIters=400, flexibleCG=1, seed=2)
    s.set_mesh(xyz, conn, lab)
    s.assemble()
    rp, ci, _ = s.matrix()
    A = reference_mat_override(rp, ci, matio.read(os.path.join(ref_data, matA)))
    s.set_matrix_csr(A.indptr, A.indices, A.data)
    b = matio.read(os.path.join(ref_data, matb))
    x, st = s.solve(b)
    assert st["status"] == 0
    assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) <= 1.05e-8
    xa = matio.read(os.path.join(ref_data, ans))
    assert np.linalg.norm(x - xa) < tol


def test_error_paths():
    s = femgpu.Solver()
    xyz, conn = meshes.kuhn_cube(3)
    bad = conn.copy()
    bad[0, 0] = 10**6
    with pytest.raises(femgpu.FemgpuError) as e:
        s.set_mesh(xyz, bad)
    assert e.value.status == 1
    with pytest.raises(femgpu.FemgpuError) as e:
        s.setup()
    assert e.value.status == 3
    rp = np.array([0, 2, 3], np.int32)
    with pytest.raises(femgpu.FemgpuError) as e:
        s.set_matrix_csr(rp, np.array([1, 0, 1], np.int32), np.ones(3))
    assert e.value.status == 1
    # maxIters reached is reported, not hidden
    s2 = femgpu.Solver(solverType=1, tolerance=1e-14, maxIters=2, seed=1)
    xyz, conn, kappa, f, mask = meshes.poisson3d_problem(8)
    s2.set_mesh(xyz, conn)
    s2.assemble(kappa, 0.0)
    s2.set_dirichlet(mask)
    x, st = s2.solve(s2.load_vector(f), check=False)
    assert st["status"] == 5 and st["iterations"] == 2


def test_native_library_is_the_cuda_path():
    launches0 = femgpu.kernel_launches()
    s, _ = gpu_operator(*meshes.kuhn_cube(4))
    assert femgpu.kernel_launches() > launches0
    assert femgpu.native_library_path().endswith("libfemgpu.so")


@pytest.mark.parametrize("cycle,n", [(1, 40), (2, 40), (1, 64), (2, 64)])
def test_w_and_f_cycles_match_oracle(cycle, n):
    # W- and F-cycles: the next coarser level visited twice (second visit on the coarse
    # residual); the cycle and the PCG against the oracle with the same cycle type
    xyz, conn, kappa, f, mask = meshes.poisson3d_problem(n, sigma=2.0)
    rp, ci, v, b = oracle_operator(xyz, conn, coef=kappa, lam=0.0, mask=mask, f=f)
    gx, ga = meshes.adjacency_from_pattern(rp, ci)
    orc = O.OracleAMG(rp, ci, v, gx, ga, seed=5, cycle_type=cycle)
    s, gb = gpu_operator(xyz, conn, coef=kappa, lam=0.0, mask=mask, f=f, seed=5, cycleType=cycle,
                         solverType=1, tolerance=1e-8, maxIters=300, flexibleCG=1)
    s.setup()
    assert s.num_levels == orc.num_levels >= 3
    r = np.random.default_rng(0).standard_normal(rp.shape[0] - 1)
    zg, zo = s.vcycle(r), orc.vcycle(r)
    assert np.array_equal(zg, zo), np.abs(zg - zo).max() / np.abs(zo).max()
    x, st = s.solve(b)
    xo, sto = orc.pcg(b, tol=1e-8, max_iters=300, flexible=True)
    assert st["status"] == 0 and abs(st["iterations"] - sto["iters"]) <= 1
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-8
    # the V-cycle of the same hierarchy differs: the second visits change the result
    s.set_config(cycleType=0)
    assert not np.array_equal(s.vcycle(r), zg)


def test_cycle_type_is_validated():
    with pytest.raises(femgpu.FemgpuError):
        femgpu.Solver(cycleType=3)


@pytest.mark.parametrize("n", [40, 64])
def test_autotuned_launch_choices_keep_every_bit(n, tmp_path, monkeypatch):
    # the autotuner only picks launch shapes that leave every sum unchanged: a tuned and an
    # untuned handle give the same V-cycle and the same PCG iterates bit for bit
    monkeypatch.setenv("FEMGPU_TUNE_CACHE", str(tmp_path / "tune.txt"))
    xyz, conn, kappa, f, mask = meshes.poisson3d_problem(n, sigma=2.0)
    runs = []
    for tune in (1, 0):
        s, b = gpu_operator(xyz, conn, coef=kappa, lam=0.0, mask=mask, f=f, seed=5, autotune=tune,
                            solverType=1, tolerance=1e-8, maxIters=300, flexibleCG=1)
        s.setup()
        r = np.random.default_rng(0).standard_normal(s.n)
        runs.append((s.vcycle(r), s.solve(b)))
    (z1, (x1, st1)), (z0, (x0, st0)) = runs
    assert np.array_equal(z1, z0)
    assert np.array_equal(x1, x0) and st1["iterations"] == st0["iterations"]


@pytest.mark.parametrize("precision,sweeps,n", [(0, 2, 40), (1, 2, 40), (0, 3, 64)])
def test_l1_jacobi_smoother_matches_oracle(precision, sweeps, n):
    # the performance smoother (smoother = 1): l1-Jacobi sweeps on each level's whole operator;
    # the cycle bit for bit against the oracle's restatement, the PCG within 1e-8
    xyz, conn, kappa, f, mask = meshes.poisson3d_problem(n, sigma=2.0)
    rp, ci, v, b = oracle_operator(xyz, conn, coef=kappa, lam=0.0, mask=mask, f=f)
    gx, ga = meshes.adjacency_from_pattern(rp, ci)
    orc = O.OracleAMG(rp, ci, v, gx, ga, seed=5, smoother=1, pre_inner=sweeps, post_inner=sweeps,
                      fp64_hierarchy=precision)
    s, gb = gpu_operator(xyz, conn, coef=kappa, lam=0.0, mask=mask, f=f, seed=5, smoother=1, precision=precision,
                         preInnerIters=sweeps, postInnerIters=sweeps, solverType=1, tolerance=1e-8, maxIters=300,
                         flexibleCG=1)
    s.setup()
    r = np.random.default_rng(0).standard_normal(rp.shape[0] - 1)
    zg, zo = s.vcycle(r), orc.vcycle(r)
    assert np.array_equal(zg, zo), np.abs(zg - zo).max() / np.abs(zo).max()
    x, st = s.solve(b)
    xo, sto = orc.pcg(b, tol=1e-8, max_iters=300, flexible=True)
    assert st["status"] == 0 and abs(st["iterations"] - sto["iters"]) <= 1
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-8
