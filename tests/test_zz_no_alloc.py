"""femgpu_load_vector_device_noalloc against femgpu_load_vector (needs a GB300).

This file sorts last so that it also runs after every other GPU test in the same
process; it builds its own meshes and passes on its own as well.
"""
import ctypes as C

import numpy as np
import pytest

import femgpu
from femgpu import meshes

pytestmark = pytest.mark.gpu

def _header_limit():
    """FEMGPU_NOALLOC_MAX_ELEMENTS as include/femgpu.h defines it."""
    import os
    import re
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "femgpu.h")
    with open(path) as fh:
        return int(re.search(r"#define\s+FEMGPU_NOALLOC_MAX_ELEMENTS\s+(\d+)", fh.read()).group(1))


MAX_ELEMENTS = _header_limit()

# CUmemPool_attribute values from cuda.h
_USED_MEM_CURRENT = 7
_USED_MEM_HIGH = 8


class _StreamPool:
    """Usage counters of the device's current memory pool, read through the driver
    API; the solver under test is given this pool for its device buffers."""

    def __init__(self, device=0):
        self.cu = C.CDLL("libcuda.so.1")
        dev = C.c_int()
        assert self.cu.cuDeviceGet(C.byref(dev), device) == 0
        self.pool = C.c_void_p()
        assert self.cu.cuDeviceGetMemPool(C.byref(self.pool), dev) == 0

    def _get(self, attr):
        v = C.c_uint64()
        assert self.cu.cuMemPoolGetAttribute(self.pool, attr, C.byref(v)) == 0
        return v.value

    def used(self):
        return self._get(_USED_MEM_CURRENT)

    def high(self):
        return self._get(_USED_MEM_HIGH)

    def reset_high(self):
        zero = C.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, _USED_MEM_HIGH, C.byref(zero)) == 0


def _mesh_solver(kind, pool=None):
    rng = np.random.default_rng(11)
    if kind == "tet":
        xyz, conn = meshes.kuhn_cube(14)
        xyz = xyz + rng.uniform(-0.01, 0.01, xyz.shape)
    else:
        xyz, conn = meshes.jittered_square(40)
    s = femgpu.Solver(mem_pool=pool.pool.value) if pool else femgpu.Solver()
    s.set_mesh(xyz, conn)
    return s, xyz.shape[0], rng


@pytest.mark.parametrize("kind", ["tet", "tri"])
def test_two_consecutive_calls_match_allocating_entry_point(kind):
    import torch

    torch.cuda.init()
    pool = _StreamPool()
    s, nv, rng = _mesh_solver(kind, pool)
    f1 = rng.uniform(-1.0, 1.0, nv)
    f2 = rng.standard_normal(nv) * 3.0
    torch.cuda.synchronize()
    pool.reset_high()
    before_alloc = pool.used()
    ref1 = s.load_vector(f1)
    # the allocating entry point draws its buffers from this pool, so the pool sees them
    assert pool.high() > before_alloc
    ref2 = s.load_vector(f2)

    dev = torch.device("cuda", 0)
    df1 = torch.from_numpy(f1).to(dev)
    df2 = torch.from_numpy(f2).to(dev)
    db1 = torch.full((nv,), float("nan"), dtype=torch.float64, device=dev)
    db2 = torch.full((nv,), float("nan"), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()

    used0 = pool.used()
    pool.reset_high()
    launches0 = femgpu.kernel_launches()
    s.load_vector_device_noalloc(df1.data_ptr(), db1.data_ptr())
    s.load_vector_device_noalloc(df2.data_ptr(), db2.data_ptr())
    torch.cuda.synchronize()
    assert femgpu.kernel_launches() - launches0 == 4
    # no allocation from the solver's pool happened inside either call
    assert pool.high() <= used0
    assert pool.used() == used0

    np.testing.assert_array_equal(db1.cpu().numpy(), ref1)
    np.testing.assert_array_equal(db2.cpu().numpy(), ref2)


def test_rejects_bad_calls_without_launching():
    import torch

    s = femgpu.Solver()
    dev = torch.device("cuda", 0)
    buf = torch.zeros(8, dtype=torch.float64, device=dev)
    launches0 = femgpu.kernel_launches()
    # no mesh yet
    assert s.load_vector_device_noalloc(buf.data_ptr(), buf.data_ptr(), check=False) == 3
    assert femgpu.kernel_launches() == launches0
    # null device pointers
    s2, nv, _ = _mesh_solver("tri")
    launches1 = femgpu.kernel_launches()
    assert s2.load_vector_device_noalloc(0, buf.data_ptr(), check=False) == 1
    assert femgpu.kernel_launches() == launches1
    # more elements than the fixed scratch holds: the smallest Kuhn cube above the limit
    cells = 1
    while 6 * cells ** 3 <= MAX_ELEMENTS:
        cells += 1
    xyz, conn = meshes.kuhn_cube(cells)
    assert conn.shape[0] > MAX_ELEMENTS
    big = femgpu.Solver()
    big.set_mesh(xyz, conn)
    f = torch.zeros(xyz.shape[0], dtype=torch.float64, device=dev)
    b = torch.full((xyz.shape[0],), 7.0, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    before = femgpu.kernel_launches()
    assert big.load_vector_device_noalloc(f.data_ptr(), b.data_ptr(), check=False) == 6
    assert femgpu.kernel_launches() == before
    torch.cuda.synchronize()
    assert bool((b == 7.0).all())
