"""C ABI surface and host-side logic (runs without a GPU: no compute calls)."""
import ctypes
import os
import re

import numpy as np
import pytest

import matio
from conftest import ROOT, gpu_available

import femgpu
from femgpu import capi


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "femgpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(femgpu_[a-z_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = capi.lib()
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(capi.EXPORTS) == syms


def test_library_is_built_for_sm103a():
    # the shared library is in-tree and was built by nvcc for sm_103a only
    path = capi.native_library_path()
    assert path.startswith(os.path.join(ROOT, "sci-solver_fem_gb300"))
    from femgpu import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_config_defaults_match_femsolver():
    c = capi.Config()
    capi.lib().femgpu_config_default(ctypes.byref(c))
    # FEMSolver::FEMSolver defaults (src/FEMSolver.cu:9-35)
    assert (c.maxLevels, c.maxIters, c.preInnerIters, c.postInnerIters, c.postRelaxes) == (100, 100, 5, 5, 1)
    assert (c.topSize, c.randMisParameters, c.partitionMaxSize, c.aggregatorType) == (256, 90102, 512, 0)
    assert (c.tolerance, c.smootherWeight, c.proOmega, c.solverType, c.blockSize) == (1e-6, 1.0, 0.67, 0, 256)


@pytest.mark.skipif(gpu_available(), reason="checks the no-device path")
def test_create_without_device_reports_status():
    with pytest.raises(femgpu.FemgpuError) as e:
        femgpu.Solver()
    assert e.value.status == 9


def test_status_strings():
    lib = capi.lib()
    for code, name in capi.STATUS.items():
        assert lib.femgpu_status_string(code).decode() == name


def test_read_tetgen_fixture(ref_data):
    xyz, conn, lab = femgpu.read_tetgen(os.path.join(ref_data, "simple"))
    assert xyz.shape == (5000, 3) and conn.shape == (14406, 4)
    assert conn.min() == 0 and conn.max() == 4999
    # coordinates are parsed as float (tetmesh.cu:297-307)
    assert np.all(xyz.astype(np.float32).astype(np.float64) == xyz)
    xyz2, conn2, _ = femgpu.read_tetgen(os.path.join(ref_data, "CubeMesh_size256step16_correct"))
    assert xyz2.shape == (4913, 3) and conn2.shape == (24576, 4) and conn2.min() == 0


def test_read_ply_fixture(ref_data):
    xyz, tri = femgpu.read_ply(os.path.join(ref_data, "simple.ply"))
    assert xyz.shape == (2500, 3) and tri.shape == (4802, 3)
    xyz, tri = femgpu.read_ply(os.path.join(ref_data, "sphere_290verts.ply"))
    assert xyz.shape[0] == 290 and tri.max() < 290


def test_mat_readers_agree_with_numpy_reader(ref_data):
    for name in ("tetVolA.mat", "simple.mat", "simpleTri.mat"):
        rp, ci, v, shape = femgpu.read_mat_sparse(os.path.join(ref_data, name))
        A = matio.read(os.path.join(ref_data, name))
        assert shape == A.shape
        assert np.array_equal(rp, A.indptr) and np.array_equal(ci, A.indices) and np.array_equal(v, A.data)
    for name in ("tetVolb.mat", "tetVolAns.mat", "simpleb.mat", "simpleTrib.mat"):
        assert np.array_equal(femgpu.read_mat_array(os.path.join(ref_data, name)), matio.read(os.path.join(ref_data, name)))


def test_mat_write_roundtrip(tmp_path):
    v = np.linspace(-1, 1, 37)
    p = str(tmp_path / "x.mat")
    femgpu.write_mat_array(p, v)
    assert np.array_equal(femgpu.read_mat_array(p), v)
    assert np.array_equal(matio.read(p), v)


def test_vtk_writer(tmp_path):
    xyz, conn = femgpu.meshes.kuhn_cube(2)
    p = str(tmp_path / "m.vtk")
    femgpu.write_vtk(p, xyz, conn, np.arange(xyz.shape[0], dtype=float))
    txt = open(p).read()
    assert "CELLS 48 240" in txt and "POINT_DATA 27" in txt


def test_corrupt_files_return_io_status(tmp_path):
    bad = tmp_path / "bad.node"
    bad.write_text("not a node file\n")
    (tmp_path / "bad.ele").write_text("1 4 0\n1 0 1 2 3\n")
    with pytest.raises(femgpu.FemgpuError) as e:
        femgpu.read_tetgen(str(tmp_path / "bad"))
    assert e.value.status == 7
    (tmp_path / "bad.mat").write_bytes(b"\0" * 200)
    with pytest.raises(femgpu.FemgpuError) as e:
        femgpu.read_mat_sparse(str(tmp_path / "bad.mat"))
    assert e.value.status == 7
    with pytest.raises(femgpu.FemgpuError):
        femgpu.read_ply(str(tmp_path / "missing.ply"))


def test_ply_coordinates_keep_their_stored_precision(tmp_path):
    # ASCII values are scanned as double (the reference's TriMesh reader uses "%lf");
    # binary float and double properties keep their stored values
    xyz = np.array([[0.1, 0.2, 0.0], [1.0 / 3.0, 0.7, 0.0], [0.9, 0.123456789012345, 0.0]])
    faces = np.array([[0, 1, 2]], np.int32)
    asc = tmp_path / "a.ply"
    with open(asc, "w") as f:
        f.write("ply\nformat ascii 1.0\nelement vertex 3\nproperty double x\nproperty double y\n"
                "property double z\nelement face 1\nproperty list uchar int vertex_indices\nend_header\n")
        for p in xyz:
            f.write(" ".join(repr(float(c)) for c in p) + "\n")
        f.write("3 0 1 2\n")
    got, tri = femgpu.read_ply(str(asc))
    assert np.array_equal(got, xyz) and np.array_equal(tri, faces)
    for typ, dt in (("double", "<f8"), ("float", "<f4")):
        b = tmp_path / f"b_{typ}.ply"
        with open(b, "wb") as f:
            f.write((f"ply\nformat binary_little_endian 1.0\nelement vertex 3\nproperty {typ} x\n"
                     f"property {typ} y\nproperty {typ} z\nelement face 1\n"
                     "property list uchar int vertex_indices\nend_header\n").encode())
            f.write(xyz.astype(dt).tobytes())
            f.write(np.array([3], np.uint8).tobytes() + faces.astype("<i4").tobytes())
        got, tri = femgpu.read_ply(str(b))
        assert np.array_equal(got, xyz.astype(dt).astype(np.float64)) and np.array_equal(tri, faces)
