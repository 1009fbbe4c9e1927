"""Pins the mesh readers and the sparsity patterns to the reference's own code (no GPU).

The reference's TetMesh reader and vertex-neighbour builder (src/core/cuda/tetmesh.cu,
TetMesh::read :251-376 and need_neighbors :112-170) and its TriMesh PLY reader and
neighbour builder (src/core/aggmis/cuda/TriMesh_io.cu, TriMesh_connectivity.cu) have no
CUSP dependency, so oracle/ref.mk compiles them from the reference sources into
oracle/_ref/.  The pattern the reference builds from them (tetmesh2ell and trimesh2ell,
src/core/cuda/cutil.cu:169-230,297-348) is row i = [i, sorted neighbours of i]; this
repository stores the same columns in ascending order.  Skipped where the reference
checkout is absent (the library is built from its sources).
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import femgpu
import oracle as O
from femgpu import meshes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("FEMGPU_REFERENCE", "/root/reference")
LIB = os.path.join(ROOT, "oracle", "_ref", "libref_tetmesh.so")


@pytest.fixture(scope="module")
def ref():
    if not os.path.exists(LIB):
        if not os.path.isdir(os.path.join(REF, "src", "core")):
            pytest.skip("the reference checkout is not on this machine")
        subprocess.run(["make", "-s", "-f", os.path.join(ROOT, "oracle", "ref.mk"), f"REF={REF}"], check=True)
    L = C.CDLL(LIB)
    L.ref_tetmesh_read.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.ref_tetmesh_arrays.argtypes = [C.c_void_p, C.c_void_p]
    L.ref_tetmesh_neighbors.argtypes = [C.c_void_p, C.c_void_p]
    L.ref_tetmesh_neighbors.restype = C.c_int64
    L.ref_trimesh_read.argtypes = [C.c_char_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.ref_trimesh_arrays.argtypes = [C.c_void_p, C.c_void_p]
    L.ref_trimesh_neighbors.argtypes = [C.c_void_p, C.c_void_p]
    L.ref_trimesh_neighbors.restype = C.c_int64
    return L


def reference_mesh(L, base):
    nv, ne = C.c_int64(), C.c_int64()
    assert L.ref_tetmesh_read((base + ".node").encode(), (base + ".ele").encode(), C.byref(nv), C.byref(ne)) == 0
    xyz = np.zeros((nv.value, 3))
    tets = np.zeros((ne.value, 4), np.int32)
    L.ref_tetmesh_arrays(xyz.ctypes.data, tets.ctypes.data)
    off = np.zeros(nv.value + 1, np.int32)
    total = L.ref_tetmesh_neighbors(off.ctypes.data, None)
    nbr = np.zeros(max(total, 1), np.int32)
    L.ref_tetmesh_neighbors(off.ctypes.data, nbr.ctypes.data)
    return xyz, tets, off, nbr[:total]


def write_tetgen(base, xyz, conn, one_based=True):
    o = 1 if one_based else 0
    with open(base + ".node", "w") as f:
        f.write(f"{xyz.shape[0]} 3 0 0\n")
        for i, p in enumerate(xyz):
            f.write(f"{i + o} {p[0]:.9g} {p[1]:.9g} {p[2]:.9g}\n")
    with open(base + ".ele", "w") as f:
        f.write(f"{conn.shape[0]} 4 0\n")
        for e, t in enumerate(conn):
            f.write(f"{e + o} {t[0] + o} {t[1] + o} {t[2] + o} {t[3] + o}\n")


def cases(tmp_path_factory, ref_data):
    d = tmp_path_factory.mktemp("meshes")
    out = [os.path.join(ref_data, "tetVol"), os.path.join(ref_data, "CubeMesh_size256step16_correct"),
           os.path.join(ref_data, "simple")]
    xyz, conn = meshes.kuhn_cube(7)
    rng = np.random.default_rng(3)
    xyz = xyz + rng.uniform(-0.02, 0.02, xyz.shape)
    write_tetgen(str(d / "kuhn7"), xyz, conn, one_based=True)
    write_tetgen(str(d / "kuhn5z"), *meshes.kuhn_cube(5), one_based=False)
    return out + [str(d / "kuhn7"), str(d / "kuhn5z")]


def test_reader_and_pattern_match_the_reference(ref, tmp_path_factory, ref_data):
    for base in cases(tmp_path_factory, ref_data):
        rxyz, rtets, off, nbr = reference_mesh(ref, base)
        xyz, conn, _ = femgpu.read_tetgen(base)
        # the same vertices (bit for bit) and elements
        assert np.array_equal(xyz, rxyz), base
        assert np.array_equal(conn, rtets), base
        # the pattern: every row's columns are the vertex and its reference neighbours
        rp, ci = O.build_pattern(xyz.shape[0], conn)
        for i in range(xyz.shape[0]):
            want = np.unique(np.concatenate([[i], nbr[off[i]:off[i + 1]]]))
            assert np.array_equal(ci[rp[i]:rp[i + 1]], want), (base, i)
        # need_neighbors lists each neighbour once
        for i in range(xyz.shape[0]):
            row = nbr[off[i]:off[i + 1]]
            assert len(np.unique(row)) == len(row), (base, i)


def reference_trimesh(L, path):
    nv, nf = C.c_int64(), C.c_int64()
    assert L.ref_trimesh_read(path.encode(), C.byref(nv), C.byref(nf)) == 0
    xyz = np.zeros((nv.value, 3))
    faces = np.zeros((nf.value, 3), np.int32)
    L.ref_trimesh_arrays(xyz.ctypes.data, faces.ctypes.data)
    off = np.zeros(nv.value + 1, np.int32)
    total = L.ref_trimesh_neighbors(off.ctypes.data, None)
    nbr = np.zeros(max(total, 1), np.int32)
    L.ref_trimesh_neighbors(off.ctypes.data, nbr.ctypes.data)
    return xyz, faces, off, nbr[:total]


def write_ply(path, xyz, faces):
    with open(path, "w") as f:
        f.write("ply\nformat ascii 1.0\n")
        f.write(f"element vertex {xyz.shape[0]}\nproperty float x\nproperty float y\nproperty float z\n")
        f.write(f"element face {faces.shape[0]}\nproperty list uchar int vertex_indices\nend_header\n")
        for p in xyz:
            f.write(f"{p[0]:.7g} {p[1]:.7g} {p[2]:.7g}\n")
        for t in faces:
            f.write(f"3 {t[0]} {t[1]} {t[2]}\n")


def test_ply_reader_and_pattern_match_the_reference(ref, tmp_path, ref_data):
    xyz2, tri2 = meshes.jittered_square(24, seed=5)
    xyz3 = np.zeros((xyz2.shape[0], 3))
    xyz3[:, : xyz2.shape[1]] = xyz2[:, :3] if xyz2.shape[1] >= 3 else xyz2
    write_ply(str(tmp_path / "square24.ply"), xyz3, tri2)
    for path in (os.path.join(ref_data, "simple.ply"), os.path.join(ref_data, "sphere_290verts.ply"),
                 str(tmp_path / "square24.ply")):
        rxyz, rfaces, off, nbr = reference_trimesh(ref, path)
        xyz, conn = femgpu.read_ply(path)
        assert np.array_equal(xyz, rxyz), path
        assert np.array_equal(conn, rfaces), path
        rp, ci = O.build_pattern(xyz.shape[0], conn)
        for i in range(xyz.shape[0]):
            want = np.unique(np.concatenate([[i], nbr[off[i]:off[i + 1]]]))
            assert np.array_equal(ci[rp[i]:rp[i + 1]], want), (path, i)
