"""AMG hierarchy written to a file and read back in place of setup (needs a GB300).

A handle that loads the hierarchy of another handle with the same operator must solve
bit-identically to it; a file for another operator, another precision, or a damaged file
is refused."""
import numpy as np
import pytest

import femgpu
from femgpu import meshes

pytestmark = pytest.mark.gpu


def make(n=10, sigma=2.0, precision=0, kappa_seed=2):
    xyz, conn, kappa, f, mask = meshes.poisson3d_problem(n, sigma=sigma, kappa_seed=kappa_seed)
    s = femgpu.Solver(solverType=1, tolerance=1e-10, maxIters=500, flexibleCG=1, seed=4, precision=precision)
    s.set_mesh(xyz, conn)
    s.assemble(kappa, 0.0)
    s.set_dirichlet(mask)
    b = np.where(mask.astype(bool), 0.0, s.load_vector(f))
    return s, b


@pytest.mark.parametrize("precision", [0, 1])
def test_loaded_hierarchy_solves_identically(tmp_path, precision):
    path = str(tmp_path / "h.bin")
    a, b = make(precision=precision)
    a.setup()
    xa, sta = a.solve(b)
    a.save_hierarchy(path)
    c, b2 = make(precision=precision)
    c.load_hierarchy(path)
    assert c.num_levels == a.num_levels
    xc, stc = c.solve(b2)
    assert np.array_equal(xa, xc) and sta["iterations"] == stc["iterations"]
    for l in range(a.num_levels - 1):
        la, lc = a.level(l), c.level(l)
        for k in ("perm", "agg_idx", "part_idx", "P_rowptr", "P_cols", "P_vals", "A_vals"):
            assert np.array_equal(la[k], lc[k]), (l, k)


def test_load_refuses_other_operator_precision_and_damage(tmp_path):
    path = str(tmp_path / "h.bin")
    a, b = make(n=8)
    a.setup()
    a.save_hierarchy(path)
    other, _ = make(n=8, kappa_seed=3)  # same pattern, other coefficients
    assert other.load_hierarchy(path, check=False) == 1  # FEMGPU_ERR_INVALID
    fp64, _ = make(n=8, precision=1)
    assert fp64.load_hierarchy(path, check=False) == 1
    data = open(path, "rb").read()
    cut = tmp_path / "cut.bin"
    cut.write_bytes(data[: len(data) // 2])
    same, b2 = make(n=8)
    assert same.load_hierarchy(str(cut), check=False) == 7  # FEMGPU_ERR_IO
    junk = tmp_path / "junk.bin"
    junk.write_bytes(b"not a hierarchy" * 10)
    assert same.load_hierarchy(str(junk), check=False) == 7
    assert same.load_hierarchy(str(tmp_path / "missing.bin"), check=False) == 7
    # the handle is still usable: a good file, then a solve equal to the writer's
    same.load_hierarchy(path)
    x1, _ = same.solve(b2)
    x0, _ = a.solve(b)
    assert np.array_equal(x0, x1)
