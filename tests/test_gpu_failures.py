"""Failure detection on the GPU path, in forms that fault or hang nothing (needs a GB300).

* A bounded wait that runs out: the level-0 register smoother is told to give up on its
  staged-entry copies at once; the solve reports FEMGPU_ERR_LIMIT, and the same handle
  solves normally (bit for bit like a fresh handle) once the limit is restored.
* Breakdown: a NaN in the right-hand side, and a negative definite operator (every
  diagonal entry negative), each end the PCG with FEMGPU_ERR_BREAKDOWN.
* Allocation failure: a memory pool capped below what the problem needs gives
  FEMGPU_ERR_ALLOC, not a crash.
* Loop caps: isolated vertices (rows with only a diagonal) never join an aggregate; the
  aggregation loop stops at its cap with FEMGPU_ERR_LIMIT (the CPU oracle does the same).
"""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

import femgpu
import oracle as O
from femgpu import meshes

pytestmark = pytest.mark.gpu


def poisson(n=10, **opts):
    xyz, conn, kappa, f, mask = meshes.poisson3d_problem(n, sigma=2.0)
    s = femgpu.Solver(solverType=1, tolerance=1e-8, maxIters=300, flexibleCG=1, seed=3, **opts)
    s.set_mesh(xyz, conn)
    s.assemble(kappa, 0.0)
    s.set_dirichlet(mask)
    b = np.where(mask.astype(bool), 0.0, s.load_vector(f))
    return s, b


def test_copy_wait_running_out_reports_limit_and_handle_recovers():
    s, b = poisson()
    s.setup()
    s.test_copy_wait_limit(0)
    x, st = s.solve(b, check=False)
    assert st["status"] == 6  # FEMGPU_ERR_LIMIT
    assert "wait ran out" in femgpu.capi.lib().femgpu_last_error(s.h).decode()
    with pytest.raises(femgpu.FemgpuError) as e:
        s.vcycle(b)
    assert e.value.status == 6
    s.test_copy_wait_limit(-1)
    x1, st1 = s.solve(b)
    fresh, b2 = poisson()
    x2, st2 = fresh.solve(b2)
    assert st1["status"] == 0 and np.array_equal(x1, x2) and st1["iterations"] == st2["iterations"]


def test_nan_in_right_hand_side_is_breakdown():
    s, b = poisson(8)
    b = b.copy()
    b[17] = np.nan
    x, st = s.solve(b, check=False)
    assert st["status"] == 4  # FEMGPU_ERR_BREAKDOWN


def test_negative_definite_operator_is_breakdown():
    s, b = poisson(8)
    rp, ci, v = s.matrix()
    neg = femgpu.Solver(solverType=1, tolerance=1e-8, maxIters=300, flexibleCG=1, seed=3)
    neg.set_matrix_csr(rp, ci, -v)
    x, st = neg.solve(b, check=False)
    assert st["status"] == 4 and st["iterations"] <= 1


class _CappedPool:
    """A device memory pool whose size is capped (driver API cuMemPoolCreate, maxSize)."""

    class _Loc(C.Structure):
        _fields_ = [("type", C.c_int), ("id", C.c_int)]

    class _Props(C.Structure):
        pass

    _Props._fields_ = [("allocType", C.c_int), ("handleTypes", C.c_int), ("location", _Loc),
                       ("win32SecurityAttributes", C.c_void_p), ("maxSize", C.c_size_t), ("usage", C.c_ushort),
                       ("reserved", C.c_ubyte * 54)]

    def __init__(self, max_bytes, device=0):
        self.cu = C.CDLL("libcuda.so.1")
        props = self._Props()
        props.allocType = 1  # CU_MEM_ALLOCATION_TYPE_PINNED
        props.handleTypes = 0  # CU_MEM_HANDLE_TYPE_NONE
        props.location = self._Loc(1, device)  # CU_MEM_LOCATION_TYPE_DEVICE
        props.maxSize = max_bytes
        self.pool = C.c_void_p()
        assert self.cu.cuMemPoolCreate(C.byref(self.pool), C.byref(props)) == 0

    def close(self):
        if self.pool:
            self.cu.cuMemPoolDestroy(self.pool)
            self.pool = None


def test_capped_memory_pool_reports_alloc():
    torch = pytest.importorskip("torch")
    torch.cuda.init()
    femgpu.Solver().close()  # the runtime has a current context for the driver calls below
    pool = _CappedPool(4 << 20)
    try:
        xyz, conn, kappa, f, mask = meshes.poisson3d_problem(30, sigma=1.0)
        s = femgpu.Solver(solverType=1, tolerance=1e-8, mem_pool=pool.pool.value)
        with pytest.raises(femgpu.FemgpuError) as e:
            s.set_mesh(xyz, conn)
            s.assemble(kappa, 0.0)
            s.setup()
        assert e.value.status == 8  # FEMGPU_ERR_ALLOC
        assert "cudaMallocAsync" in str(e.value)
        s.close()
    finally:
        pool.close()
    # the device is fine: an uncapped handle solves as usual
    s2, b2 = poisson(6)
    x, st = s2.solve(b2)
    assert st["status"] == 0


def test_isolated_vertices_stop_the_aggregation_loop_at_its_cap():
    xyz, conn, kappa, f, mask = meshes.poisson3d_problem(6)
    rp, ci = O.build_pattern(xyz.shape[0], conn)
    v = O.assemble(xyz, conn, rp, ci, coef=kappa, lambda_mass=0.0)
    A = sp.block_diag([sp.csr_matrix((v, ci, rp)), sp.identity(3)]).tocsr()
    A.sort_indices()
    rp2, ci2 = A.indptr.astype(np.int32), A.indices.astype(np.int32)
    gx, ga = meshes.adjacency_from_pattern(rp2, ci2)
    with pytest.raises(RuntimeError, match="status 6"):
        O.OracleAMG(rp2, ci2, A.data, gx, ga, seed=1)
    s = femgpu.Solver(solverType=1, seed=1)
    s.set_matrix_csr(rp2, ci2, A.data)
    with pytest.raises(femgpu.FemgpuError) as e:
        s.setup()
    assert e.value.status == 6  # FEMGPU_ERR_LIMIT
