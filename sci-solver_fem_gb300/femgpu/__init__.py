"""femgpu -- GB300-native P1 FEM -> smoothed-aggregation AMG -> PCG solver.

Python binding of the C ABI in include/femgpu.h (libfemgpu.so, built in-tree for
sm_103a).  There is no CPU fallback: every compute call goes to the CUDA library,
and importing the binding fails loudly when the library is missing.

Typical use (the FEMSolver flow of the reference, src/FEMSolver.cu:9-93):

    from femgpu import Solver, meshes
    xyz, conn = meshes.kuhn_cube(32)
    s = Solver(solverType=1, tolerance=1e-8)
    s.set_mesh(xyz, conn)
    s.assemble()                 # K + M with label coefficients, as the reference
    x, stats = s.solve(b)
"""
from __future__ import annotations

from .capi import (FemgpuError, Solver, native_library_path, kernel_launches, read_tetgen, read_ply,
                   read_mat_sparse, read_mat_array, write_mat_array, write_vtk, STATUS, solve_batch)
from . import meshes

__all__ = ["FemgpuError", "Solver", "meshes", "native_library_path", "kernel_launches", "read_tetgen",
           "read_ply", "read_mat_sparse", "read_mat_array", "write_mat_array", "write_vtk", "STATUS", "solve_batch"]
