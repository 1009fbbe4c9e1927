"""The example command-line program (sci-solver_fem_gb300/examples/fem_solve.cpp), the
counterpart of the reference's src/examples/example1.cu and example2.cu, built against the
FEMSolver drop-in.  Building and argument handling run on the CPU; the solves need a GB300."""
import os
import subprocess

import numpy as np
import pytest

from conftest import REF_DATA, ROOT
from femgpu import capi
import matio


def build(tmp_path):
    lib = capi.native_library_path()
    exe = str(tmp_path / "fem_solve")
    src = os.path.join(ROOT, "sci-solver_fem_gb300", "examples", "fem_solve.cpp")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), src, lib, "-o", exe,
                    f"-Wl,-rpath,{os.path.dirname(lib)}"], check=True)
    return exe


def test_example_builds_and_checks_arguments(tmp_path):
    exe = build(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "-i" in r.stderr
    r = subprocess.run([exe, "-q"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "usage" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("mesh,A,b,ans,bound,vtk", [
    ("tetVol", "tetVolA.mat", "tetVolb.mat", "tetVolAns.mat", 25.0, "tetVol.vtk"),       # example1 / tetVol.cc
    ("simple.ply", "simpleTri.mat", "simpleTrib.mat", "simpleTriAns.mat", 100.0, "simple.vtk"),  # example2 / sanity2D.cc
])
def test_example_solves_reference_data(tmp_path, mesh, A, b, ans, bound, vtk):
    exe = build(tmp_path)
    r = subprocess.run([exe, "-i", os.path.join(REF_DATA, mesh), "-A", os.path.join(REF_DATA, A), "-b",
                        os.path.join(REF_DATA, b), "-s", "1"], cwd=tmp_path, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    x = matio.read(str(tmp_path / "output.mat"))
    x_ans = matio.read(os.path.join(REF_DATA, ans))
    assert np.linalg.norm(x - x_ans) < bound
    assert (tmp_path / vtk).exists()


def test_reference_test_programs_build(tmp_path):
    # the reference's gtest programs restated against the drop-in (run by the GPU tests)
    lib = capi.native_library_path()
    exe = str(tmp_path / "reference_sanity")
    src = os.path.join(ROOT, "tests", "cpp", "reference_sanity.cpp")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), src, lib, "-o", exe,
                    f"-Wl,-rpath,{os.path.dirname(lib)}"], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0  # no data directory given: usage, before any device call
